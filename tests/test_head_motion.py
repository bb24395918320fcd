"""Kinematic head: roots and attached colliders follow a rigid head pose.

The reference pins roots where Hair::Hair put them (compute.comp:144 starts
at point 1) and moves only collider 0 and the head model by keyboard
translations (Scene::translateSphere, src/Scene.cpp:110-135).  With
rvh_asset_set_head_transform each step first places every root at
head * root_rest and carries colliders marked attach_to_head with the head.
CPU tests check the host helper and the oracle; GPU tests check the kernels
against the oracle's FP32 twin (exact math: bit-identical) and FP64.
"""
import numpy as np
import pytest

from conftest import rel_pos_err
from rvh import api, configs
from rvh import types as T
from rvh._lib import RvhError


def rot_y(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]], np.float64)


def translate(d):
    m = np.eye(4)
    m[:3, 3] = d
    return m


def head_pose(k):
    """A head turning about y and drifting forward: pose before step k."""
    return (translate((0.0, 0.01 * np.sin(0.3 * k), 0.004 * k)) @ rot_y(0.02 * k)).astype(np.float32)


def head_spec(n_points=16, n_strands=256, grid_res=24):
    rec, rest, p, cols = api.generate_head(seed=11, n_strands=n_strands, n_points=n_points, root_sampling=0,
                                           sort_roots=1, length_min=0.3, length_max=0.8, head_collider=1,
                                           n_ellipsoids=2, axis_min=0.2, axis_max=0.4, grid_res=grid_res,
                                           friction=0.05, repulsion=0.02, dftl_damping=0.9)
    cols[0].attach_to_head = 1          # the head sphere and one ellipsoid ride with the head
    cols[1].attach_to_head = 1
    return configs.AssetSpec(rec, rest, p, cols, n_points)


def oracle_inputs(spec, steps):
    heads = np.stack([np.asarray(head_pose(k), np.float32).T.reshape(16) for k in range(steps)])   # column-major
    rows = [[api.collider_follow(c, head_pose(k)) if c.attach_to_head else c for c in spec.colliders]
            for k in range(steps)]
    root_rest = spec.records[:, 0, :3].copy()
    return heads, rows, root_rest


# ---- host side ----------------------------------------------------------------

def test_collider_follow_identity_and_translation(librvh):
    c = api.collider_from_trs((0.3, 1.0, -0.2), (10.0, 20.0, 30.0), (0.5, 0.8, 0.4))
    c.attach_to_head = 1
    same = api.collider_follow(c, np.eye(4, dtype=np.float32))
    assert np.array_equal(np.array(same.transform), np.array(c.transform))
    for f in ("inv", "inv_trans"):   # inverted from the float transform, not from the TRS factors
        assert np.allclose(np.array(getattr(same, f)), np.array(getattr(c, f)), rtol=1e-6, atol=1e-7)
    assert same.attach_to_head == 1
    d = np.array([0.5, -0.25, 2.0])
    moved = api.collider_follow(c, translate(d).astype(np.float32))
    tm, im = np.array(moved.transform, np.float64).reshape(4, 4).T, np.array(moved.inv, np.float64).reshape(4, 4).T
    t0 = np.array(c.transform, np.float64).reshape(4, 4).T
    assert np.allclose(tm[:3, 3], t0[:3, 3] + d, atol=1e-6)
    assert np.allclose(tm[:3, :3], t0[:3, :3])
    assert np.allclose(tm @ im, np.eye(4), atol=1e-5)
    assert np.array_equal(np.array(moved.inv_trans, np.float32).reshape(4, 4), np.array(moved.inv, np.float32).reshape(4, 4).T)


def test_collider_follow_rejects_non_affine(librvh):
    c = api.collider_from_trs((0, 0, 0), (0, 0, 0), (1, 1, 1))
    bad = np.eye(4, dtype=np.float32)
    bad[3, 0] = 0.5
    with pytest.raises(RvhError):
        api.collider_follow(c, bad)


def test_translate_keeps_the_attach_flag(librvh):
    c = api.collider_from_trs((0, 0, 0), (0, 0, 0), (1, 1, 1))
    c.attach_to_head = 1
    assert api.collider_translate(c, (0.1, 0.0, 0.0)).attach_to_head == 1


# ---- oracle ---------------------------------------------------------------------

def test_oracle_translated_head_equals_translated_scene(oracle):
    """A head translated by d from the start is the same scene shifted by d."""
    spec = configs.plain_small(n_strands=64, n_points=12)
    d = np.float32([0.25, -0.5, 0.125])      # exact in binary: x + d has one rounding either way
    steps = 5
    shifted = spec.records.copy()
    shifted[:, :spec.n_points, :3] += d
    frames = [spec.frame(k) for k in range(steps)]
    cols = [spec.colliders_at(k) for k in range(steps)]
    plain = shifted.copy()
    oracle.run(plain, spec.n_points, spec.rest, spec.params, frames, cols, steps)
    moved = shifted.copy()
    heads = np.tile(translate(d).astype(np.float32).T.reshape(16), (steps, 1))
    oracle.run(moved, spec.n_points, spec.rest, spec.params, frames, cols, steps, heads=heads,
               root_rest=spec.records[:, 0, :3])
    assert np.array_equal(moved, plain)


def test_oracle_roots_follow_the_head(oracle):
    spec = head_spec(n_strands=48)
    steps = 6
    heads, rows, root_rest = oracle_inputs(spec, steps)
    st = spec.records.astype(np.float64).copy()
    frames = [spec.frame(k) for k in range(steps)]
    oracle.run(st, spec.n_points, spec.rest, spec.params, frames, rows, steps, heads=heads, root_rest=root_rest)
    last = np.asarray(head_pose(steps - 1), np.float64)
    want = (last[:3, :3] @ root_rest.astype(np.float64).T).T + last[:3, 3]
    assert np.allclose(st[:, 0, :3], want, atol=1e-6)
    # inextensibility holds with a moving root
    seg = np.linalg.norm(np.diff(st[:, :spec.n_points, :3], axis=1), axis=2)
    assert np.allclose(seg, spec.rest[:, None].astype(np.float64), atol=1e-9)


# ---- GPU ------------------------------------------------------------------------

def _gpu_plain(ctx, spec, steps):
    a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    for k in range(steps):
        a.set_head_transform(head_pose(k))
        a.step(spec.frame(k))
    return a.read()


@pytest.mark.gpu
def test_gpu_head_exact_matches_twin(gpu_ctx, oracle):
    spec = head_spec()
    steps = 10
    heads, rows, root_rest = oracle_inputs(spec, steps)
    twin = spec.records.copy()
    oracle.run(twin, spec.n_points, spec.rest, spec.params, [spec.frame(k) for k in range(steps)], rows, steps,
               heads=heads, root_rest=root_rest, threads=8)
    got = _gpu_plain(gpu_ctx, spec, steps)
    assert np.array_equal(got, twin)


@pytest.mark.gpu
def test_gpu_head_batched_matches_plain(gpu_ctx):
    specs = [head_spec(n_points=n, n_strands=ns) for n, ns in ((8, 100), (16, 300), (32, 70))]
    steps = 6
    plain = [_gpu_plain(gpu_ctx, s, steps) for s in specs]
    assets = []
    for i, s in enumerate(specs):
        a = api.Asset(gpu_ctx, s.records, s.n_points, rest=s.rest)
        a.set_params(s.params)
        a.set_colliders(s.colliders)
        assets.append(a)
    b = api.Batch(gpu_ctx, assets, lanes=8)
    for k in range(steps):
        for i, a in enumerate(assets):
            if i != 1:                      # asset 1 keeps a still head
                a.set_head_transform(head_pose(k))
        b.step([s.frame(k) for s in specs])
    for i, (a, want) in enumerate(zip(assets, plain)):
        got = a.read()
        if i == 1:
            still = _still(gpu_ctx, specs[1], steps)
            assert np.array_equal(got, still)
        else:
            assert np.array_equal(got, want)
    b.close()


def _still(ctx, spec, steps):
    a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    for k in range(steps):
        a.step(spec.frame(k))
    return a.read()


@pytest.mark.gpu
def test_gpu_head_fast_one_step_vs_fp64(gpu_ctx_fast, oracle):
    spec = head_spec()
    heads, rows, root_rest = oracle_inputs(spec, 2)
    ref = spec.records.astype(np.float64).copy()
    oracle.run(ref, spec.n_points, spec.rest, spec.params, [spec.frame(0)], rows[:1], 1, heads=heads[:1],
               root_rest=root_rest, threads=8)
    got = _gpu_plain(gpu_ctx_fast, spec, 1)
    L = spec.rest.astype(np.float64) * (spec.n_points - 1)
    mx, p99, mean = rel_pos_err(got, ref, spec.n_points, L)
    assert mx <= 1e-5, (mx, p99, mean)


@pytest.mark.gpu
def test_gpu_head_off_keeps_roots(gpu_ctx):
    spec = head_spec(n_strands=64)
    a = api.Asset(gpu_ctx, spec.records, spec.n_points, rest=spec.rest)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    a.set_head_transform(head_pose(5))
    a.step(spec.frame(0))
    r1 = a.read()[:, 0, :3].copy()
    a.set_head_transform(None)
    a.step(spec.frame(1))
    assert np.array_equal(a.read()[:, 0, :3], r1)
