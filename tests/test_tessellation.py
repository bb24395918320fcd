"""Strand tessellation (src/shaders/hair.tesc:19-20, src/shaders/hair.tese).

CPU: the oracle's restatement against the reference's own tessellation
shader, compiled as C++ with its glm (tests/golden/tess_ref_head.npz, made by
tests/golden/make_tess_golden.py; and live where the reference checkout
exists).  GPU: rvh_asset_tessellate against the oracle, bit for bit: every
table entry and every vertex operation is separately rounded in the shader's
order, and the hash's sin is a correctly rounded one on both sides.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT
from rvh import api

GOLDEN = os.path.join(ROOT, "tests", "golden")
L, S = 12, 42


def _fixture():
    return np.load(os.path.join(GOLDEN, "tess_ref_head.npz"))


def test_oracle_matches_reference_shader_golden(oracle):
    g = _fixture()
    rec = g["records"]
    out, fr = oracle.tessellate(rec, 10, L, S, sin_mode=0, frames=True)
    ref = g["vertices"]
    # v = 1 (k = S) is where the shader reads past the strand
    assert np.array_equal(out[:, :, :S].view(np.uint32), ref[:, :, :S].view(np.uint32))
    v = (np.arange(S + 1, dtype=np.float32) / np.float32(S)).astype(np.float32)
    seg = np.minimum(np.floor(v * np.float32(9)).astype(int), 8)
    ours = fr[:, seg, :, :3].reshape(rec.shape[0], S + 1, 9)
    assert np.array_equal(ours[:, :S].view(np.uint32), g["frames"][:, 0, :S].view(np.uint32))


def test_correctly_rounded_hash_matches_the_reference_almost_always(oracle):
    """The library's hash rounds a double sin once; the reference calls the C
    library's float sin.  They differ only where that sinf is not correctly
    rounded."""
    g = _fixture()
    ours = oracle.tessellate(g["records"], 10, L, S, sin_mode=1)
    same = (ours[:, :, :S] == g["vertices"][:, :, :S]).all(-1)
    assert same.mean() >= 0.9


def test_oracle_matches_reference_shader_live(oracle):
    from oracle import build_ref_tess
    if not build_ref_tess.available():
        pytest.skip("reference checkout not present")
    lib = C.CDLL(build_ref_tess.build())
    lib.ref_tess.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    rec = np.ascontiguousarray(np.load(os.path.join(GOLDEN, "ref_head.npz"))["state_10"], np.float32)
    ns = rec.shape[0]
    ref = np.zeros((ns, L, S + 1, 4), np.float32)
    lib.ref_tess(rec.ctypes.data, ns, L, S, ref.ctypes.data, None)
    out = oracle.tessellate(rec, 10, L, S, sin_mode=0)
    assert np.array_equal(out[:, :, :S].view(np.uint32), ref[:, :, :S].view(np.uint32))


def test_oracle_curve_ends_at_the_tip_and_starts_at_the_root(oracle):
    rec, _, _, _ = api.generate_head(seed=2, n_strands=20, n_points=16, root_sampling=0, sort_roots=0,
                                     length_min=0.3, length_max=0.6, head_collider=1, n_ellipsoids=0, grid_res=0,
                                     friction=0.0, repulsion=0.0, dftl_damping=0.9)
    out = oracle.tessellate(rec, 16, L, S, clump_radius=0.0, sin_mode=1)
    assert np.array_equal(out[:, :, 0, :3], np.repeat(rec[:, None, 0, :3], L, 1))
    assert np.allclose(out[:, :, S, :3], np.repeat(rec[:, None, 15, :3], L, 1), atol=1e-6)
    assert np.allclose(out[:, :, :, 3], np.linspace(0.02, 0.01, S + 1)[None, None, :], atol=1e-7)


# ---- GPU ----------------------------------------------------------------------------

def _gpu_tess(ctx, a, ns, n, desc, frames=True):
    import torch
    per = desc.n_lines * (desc.n_segments + 1)
    vert = torch.zeros((ns * per * 4,), dtype=torch.float32, device="cuda")
    fr = torch.zeros((ns * (n - 1) * 12,), dtype=torch.float32, device="cuda") if frames else None
    torch.cuda.synchronize()
    a.tessellate(vert.data_ptr(), fr.data_ptr() if frames else None, desc=desc)
    ctx.synchronize()
    v = vert.cpu().numpy().reshape(ns, desc.n_lines, desc.n_segments + 1, 4)
    f = fr.cpu().numpy().reshape(ns, n - 1, 3, 4) if frames else None
    return v, f


@pytest.mark.gpu
@pytest.mark.parametrize("n,lines,segs,clump", [(10, 12, 42, 0.5), (2, 12, 42, 0.5), (16, 5, 17, 0.3),
                                                (32, 64, 256, 0.5), (24, 1, 1, 0.5)])
def test_gpu_tessellation_bit_exact(gpu_ctx, oracle, n, lines, segs, clump):
    rec, rest, p, cols = api.generate_head(seed=n + lines, n_strands=300, n_points=n, root_sampling=0, sort_roots=1,
                                           length_min=0.3, length_max=0.9, head_collider=1, n_ellipsoids=1,
                                           axis_min=0.2, axis_max=0.4, grid_res=0, friction=0.0, repulsion=0.0,
                                           dftl_damping=0.9)
    a = api.Asset(gpu_ctx, rec, n, rest=rest)
    a.set_params(p)
    a.set_colliders(cols)
    for k in range(3):                  # curved strands, not the straight initial ones
        a.step(api.T.frame(np.float32(1.0 / 60.0), np.float32((k + 1) / 60.0)))
    state = a.read()
    desc = api.tess_desc_reference(n_lines=lines, n_segments=segs, clump_radius=clump)
    got, gfr = _gpu_tess(gpu_ctx, a, rec.shape[0], n, desc)
    want, wfr = oracle.tessellate(state, n, lines, segs, clump_radius=clump, sin_mode=1, frames=True)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), np.abs(got - want).max()
    assert np.array_equal(gfr.view(np.uint32), wfr.view(np.uint32))


@pytest.mark.gpu
def test_gpu_tessellation_after_batched_steps(gpu_ctx, oracle):
    from rvh import configs
    specs = configs.batched(n_assets=3, scale=0.01, seed=12)
    assets = []
    for s in specs:
        a = api.Asset(gpu_ctx, s.records, s.n_points, rest=s.rest)
        a.set_params(s.params)
        a.set_colliders(s.colliders)
        assets.append(a)
    b = api.Batch(gpu_ctx, assets, lanes=8)
    for k in range(3):
        b.step([s.frame(k) for s in specs])
    desc = api.tess_desc_reference()
    for a, s in zip(assets, specs):
        got, _ = _gpu_tess(gpu_ctx, a, s.n_strands, s.n_points, desc, frames=False)
        want = oracle.tessellate(a.read(), s.n_points, desc.n_lines, desc.n_segments, sin_mode=1)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    b.close()


@pytest.mark.gpu
def test_gpu_tessellation_after_head_motion(gpu_ctx, oracle):
    """A moving head moves the roots, which pick each isoline's sd profile
    (randomChoice hashes the root): the tessellation still equals the oracle's."""
    rec, rest, p, cols = api.generate_head(seed=23, n_strands=300, n_points=12, root_sampling=0, sort_roots=1,
                                           length_min=0.3, length_max=0.9, head_collider=1, n_ellipsoids=0,
                                           grid_res=0, friction=0.0, repulsion=0.0, dftl_damping=0.9)
    a = api.Asset(gpu_ctx, rec, 12, rest=rest)
    a.set_params(p)
    a.set_colliders(cols)
    for k in range(4):
        m = np.eye(4, dtype=np.float32)
        t = 0.05 * (k + 1)
        m[0, 0], m[0, 1], m[1, 0], m[1, 1] = np.cos(t), -np.sin(t), np.sin(t), np.cos(t)
        m[0, 3] = 0.1 * (k + 1)
        a.set_head_transform(m)
        a.step(api.T.frame(np.float32(1.0 / 60.0), np.float32((k + 1) / 60.0)))
    state = a.read()
    assert not np.array_equal(state[:, 0], rec[:, 0])   # the roots moved
    desc = api.tess_desc_reference()
    got, gfr = _gpu_tess(gpu_ctx, a, rec.shape[0], 12, desc)
    want, wfr = oracle.tessellate(state, 12, desc.n_lines, desc.n_segments, sin_mode=1, frames=True)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(gfr.view(np.uint32), wfr.view(np.uint32))
    a.close()


@pytest.mark.gpu
def test_gpu_tessellation_profile_cache_follows_the_roots(gpu_ctx, oracle):
    """The sd profiles are cached per strand with the root bits they were
    computed from.  Across calls, a moving head, a write that moves a few roots
    and descriptor changes, every call still equals the oracle bit for bit."""
    rec, rest, p, cols = api.generate_head(seed=29, n_strands=400, n_points=10, root_sampling=0, sort_roots=1,
                                           length_min=0.3, length_max=0.9, head_collider=1, n_ellipsoids=0,
                                           grid_res=0, friction=0.0, repulsion=0.0, dftl_damping=0.9)
    a = api.Asset(gpu_ctx, rec, 10, rest=rest)
    a.set_params(p)
    a.set_colliders(cols)
    ref = api.tess_desc_reference()
    few = api.tess_desc_reference(n_lines=5, n_segments=17)

    def check(desc):
        got, _ = _gpu_tess(gpu_ctx, a, rec.shape[0], 10, desc, frames=False)
        want = oracle.tessellate(a.read(), 10, desc.n_lines, desc.n_segments, sin_mode=1)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        return got

    first = check(ref)
    assert np.array_equal(check(ref).view(np.uint32), first.view(np.uint32))   # cached: same bits
    for k in range(2):
        m = np.eye(4, dtype=np.float32)
        m[1, 3] = 0.07 * (k + 1)
        a.set_head_transform(m)
        a.step(api.T.frame(np.float32(1.0 / 60.0), np.float32((k + 1) / 60.0)))
        check(ref)
    a.set_head_transform(None)
    state = a.read()
    state[5, 0, :3] += np.float32(0.3)
    state[17, 0, 0] = np.float32(5.0)
    state[200, 0, 2] = np.float32(-1.25)
    a.write(state)
    check(ref)
    check(few)
    check(ref)
    a.close()


@pytest.mark.gpu
def test_gpu_tessellation_rejects_bad_descriptors(gpu_ctx):
    from rvh._lib import RvhError
    rec, rest, p, cols = api.generate_head(seed=1, n_strands=8, n_points=8, root_sampling=0, sort_roots=0,
                                           length_min=0.3, length_max=0.5, head_collider=0, n_ellipsoids=0,
                                           grid_res=0, friction=0.0, repulsion=0.0, dftl_damping=0.9)
    a = api.Asset(gpu_ctx, rec, 8, rest=rest)
    for kw in ({"n_lines": 0}, {"n_lines": 65}, {"n_segments": 0}, {"n_segments": 257}):
        with pytest.raises(RvhError):
            a.tessellate(0, None, desc=api.tess_desc_reference(**kw))
