"""Host-side pieces of the boundary: collider construction (vs the reference's
glm), reference constants, initial strands, seeded generators.  CPU only."""
import numpy as np
import pytest

from conftest import golden
from rvh import api, configs
from rvh import types as T


def flat48(c):
    return np.concatenate([np.array(c.transform), np.array(c.inv), np.array(c.inv_trans)]).astype(np.float64)


def test_collider_from_trs_matches_glm(librvh):
    g = golden("colliders.npz")
    for spec, mats in zip(g["specs"], g["mats"]):
        c = api.collider_from_trs(spec[0], spec[1], spec[2])
        got = flat48(c)
        ref = mats.astype(np.float64)
        assert np.allclose(got, ref, rtol=0, atol=2e-6 * max(1.0, np.abs(ref).max())), np.abs(got - ref).max()


def test_collider_translate_matches_translate_sphere(librvh):
    g = golden("colliders.npz")
    c = T.collider_from_flat48(g["mats"][0], T.COLLIDER_SPHERE, 1.0)
    moved = api.collider_translate(c, g["move"])
    assert np.allclose(flat48(moved), g["sphere_moved"], atol=1e-6)
    assert moved.kind == T.COLLIDER_SPHERE and moved.radius == 1.0


def test_reference_params_are_the_shader_constants(librvh):
    p = api.reference_params()
    assert tuple(p.gravity) == (0.0, np.float32(-9.8), 0.0)
    assert np.float32(p.damping) == np.float32(0.998) and np.float32(p.dftl_damping) == np.float32(0.998)
    assert p.vmax == 10.0 and p.k_penalty == 1900.0 and np.float32(p.friction) == np.float32(0.08)
    assert p.grid_scale == 1e6 and tuple(p.grid_dims) == (64, 64, 64) and p.grid_wrap32 == 1
    assert tuple(p.grid_origin) == (-3.0, -2.0, -5.0) and p.grid_h == np.float32(7.0) / np.float32(64.0)
    py = T.reference_params()
    assert bytes(py) == bytes(p)


def test_init_strands_reference_formula(librvh):
    roots = np.array([[0.0, 2.0, 0.0], [0.5, 2.5, -0.1]], np.float32)
    nrm = np.array([[0.0, 1.0, 0.0], [0.6, 0.8, 0.0]], np.float32)
    seg = np.float32(2.5) / np.float32(9.0)
    out = api.init_strands_reference(roots, nrm, 10, seg)
    for s in range(2):
        d = nrm[s] + np.array([0.05, 5.0, -2.0], np.float32)
        p = roots[s].copy()
        for j in range(10):
            assert np.array_equal(out[s, j, :3], p) and out[s, j, 3] == 1.0
            assert tuple(out[s, 10 + j]) == (0.0, 0.0, -1.0, 0.0)
            assert not out[s, 20 + j].any()
            p = (p + seg * d).astype(np.float32)


def test_generate_head_is_seeded_and_well_formed(librvh):
    a = configs.full_head(n_strands=3000, n_points=16, seed=5)
    b = configs.full_head(n_strands=3000, n_points=16, seed=5)
    c = configs.full_head(n_strands=3000, n_points=16, seed=6)
    assert np.array_equal(a.records, b.records) and not np.array_equal(a.records, c.records)
    roots = a.records[:, 0, :3].astype(np.float64)
    assert np.allclose(np.linalg.norm(roots, axis=1), 1.0, atol=1e-6) and roots[:, 1].min() >= 0.0
    L = a.rest * 15
    assert L.min() >= 0.4 - 1e-6 and L.max() <= 0.8 + 1e-6
    seg = np.linalg.norm(np.diff(a.records[:, :16, :3].astype(np.float64), axis=1), axis=2)
    assert np.allclose(seg, a.rest[:, None], rtol=1e-5)
    # Poisson-disk: no two roots closer than the dart radius (shrinks only if saturated)
    from scipy.spatial import cKDTree
    dmin = cKDTree(roots).query(roots, k=2)[0][:, 1].min()
    assert dmin > 0.5 * 0.8 * np.sqrt(4.376 / 3000)
    # grid covers the reachable region (head radius + longest strand)
    p = a.params
    assert p.grid_enabled == 1 and tuple(p.grid_dims) == (64, 64, 64)
    lo = np.array(p.grid_origin)
    hi = lo + p.grid_h * 64
    assert np.all(lo <= -1.8) and np.all(hi >= 1.8)
    assert len(a.colliders) == 5 and a.colliders[0].kind == T.COLLIDER_SPHERE
    assert all(c.kind == T.COLLIDER_ELLIPSOID for c in a.colliders[1:])


def test_plain_small_matches_its_description(librvh):
    s = configs.plain_small()
    assert s.records.shape == (1024, 48, 4) and np.allclose(s.rest, np.float32(0.5) / 15)
    assert s.params.grid_enabled == 0 and np.float32(s.params.dftl_damping) == np.float32(0.9)
    f = s.frame(59)
    assert f.dt == np.float32(1 / 60) and np.isclose(f.wind[0], 2.0 * np.sin(0.5 * f.t), atol=1e-6)
    cols = s.colliders_at(59)
    assert len(cols) == 2 and cols[1].kind == T.COLLIDER_SPHERE and np.isclose(cols[1].radius, 0.3)
    cen = np.array(cols[1].transform[12:15])
    assert np.isclose(np.hypot(cen[0], cen[2]), 1.2, atol=1e-5) and cen[1] == 0.0
    # initial direction = outward normal
    d = s.records[:, 1, :3] - s.records[:, 0, :3]
    assert np.allclose(d / np.linalg.norm(d, axis=1, keepdims=True), s.records[:, 0, :3], atol=1e-5)


def test_wind_gusts_statistics(librvh):
    w = api.WindDesc()
    w.amplitude, w.omega, w.gust_sigma, w.seed = 0.0, 0.5, 0.5, 42
    w.dir[:] = (1.0, 0.0, 0.0)
    g = np.array([api.wind_at(w, k, 0.0) for k in range(20000)])
    assert abs(g.mean()) < 0.02 and abs(g.std() - 0.5) < 0.02
    assert api.wind_at(w, 7, 1.0) == api.wind_at(w, 7, 1.0)


def test_batched_sizes_follow_the_distribution():
    sz = configs.batched_sizes()
    ns = np.array([s[0] for s in sz])
    assert len(sz) == 256 and ns.min() >= 512 and ns.max() <= 65536
    assert set(s[1] for s in sz) <= {8, 16, 24, 32} and all(32 <= s[2] <= 64 for s in sz)
    assert all(0 <= s[3] <= 4 for s in sz)
    assert 0.25 < np.mean(np.log(ns) < np.log(512 * 16)) < 0.75   # log-uniform median ~ 5.8k


def test_rng_is_counter_based(librvh):
    a = [librvh.rvh_rng_u64(3, i) for i in range(5)]
    b = [librvh.rvh_rng_u64(3, i) for i in range(5)]
    assert a == b and len(set(a)) == 5
    u = np.array([librvh.rvh_rng_uniform(9, i) for i in range(10000)])
    assert 0 <= u.min() and u.max() < 1 and abs(u.mean() - 0.5) < 0.02


def test_oracle_scene_generator_gives_the_library_bytes(librvh, oracle):
    """The CPU timing arm of bench.py builds its workload sample with the
    oracle's statement of the seeded generator, never mapping the CUDA
    library; it must be the same workload, byte for byte."""
    gen = oracle.SceneGen()
    lib_specs = configs.batched(indices=range(6))
    ora_specs = configs.batched(indices=range(6), gen=gen)
    for a, b in zip(lib_specs, ora_specs):
        assert a.records.tobytes() == b.records.tobytes()
        assert a.rest.tobytes() == b.rest.tobytes()
        assert bytes(a.params) == bytes(b.params)
        assert [bytes(c) for c in a.colliders] == [bytes(c) for c in b.colliders]
        for k in (0, 1, 57):
            assert bytes(a.frame(k)) == bytes(b.frame(k))
    kw = dict(seed=11, n_strands=3000, n_points=12, root_sampling=1, sort_roots=1, length_min=0.4,
              length_max=0.8, head_collider=1, n_ellipsoids=4, axis_min=0.2, axis_max=0.5, grid_res=40,
              friction=0.05, repulsion=0.02, dftl_damping=0.9, head_center=(0.5, -1.0, 2.0))
    x, y = api.generate_head(**kw), gen.generate_head(**kw)
    assert x[0].tobytes() == y[0].tobytes() and x[1].tobytes() == y[1].tobytes()
    assert bytes(x[2]) == bytes(y[2]) and [bytes(c) for c in x[3]] == [bytes(c) for c in y[3]]
