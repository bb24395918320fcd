"""The oracle pinned against the reference's own shader code (golden fixtures)
and against closed-form answers and the shader's invariants.  CPU only."""
import numpy as np
import pytest

from conftest import golden, rel_pos_err
from rvh import types as T

N = 10
REF_LENGTH = 2.5


def ref_frames_and_colliders(g):
    cs, times = g["colliders"], g["times"]
    steps = times.shape[0]
    frames = [T.frame(times[k, 0], times[k, 1]) for k in range(steps)]
    rows = [[T.collider_from_flat48(cs[k, j], T.COLLIDER_SPHERE if j == 0 else T.COLLIDER_ELLIPSOID, 1.0)
             for j in range(cs.shape[1])] for k in range(steps)]
    return frames, rows


def run_snapshots(oracle, g, dtype, snaps, threads=1):
    frames, rows = ref_frames_and_colliders(g)
    st = g["init"].astype(dtype)
    rest = np.full(st.shape[0], np.float32(2.5) / (np.float32(10) - np.float32(1.0)), np.float32)
    P = T.reference_params()
    out, done, grid = {}, 0, None
    for s in snaps:
        grid = oracle.run(st, N, rest, P, frames[done:s], rows[done:s], s - done, threads=threads, want_grid=True)
        done = s
        out[s] = st.copy()
    return out, grid


def wrap32(g):
    return g.astype(np.uint64).astype(np.uint32).view(np.int32)


@pytest.mark.parametrize("case,snaps", [("ref_head.npz", [1, 10, 60]), ("ref_dense.npz", [1, 2])])
@pytest.mark.parametrize("threads", [1, 4])
def test_fp32_twin_is_bit_exact_with_reference_shader(oracle, case, snaps, threads):
    g = golden(case)
    out, grid = run_snapshots(oracle, g, np.float32, snaps, threads)
    for s in snaps:
        assert np.array_equal(out[s], g["state_%d" % s]), "step %d differs" % s
    dense = np.zeros((64 ** 3, 4), np.int32)
    dense[g["grid_index"]] = g["grid_value"]
    assert np.array_equal(wrap32(grid), dense)


def test_dense_case_really_wraps(oracle):
    g = golden("ref_dense.npz")
    _, grid = run_snapshots(oracle, g, np.float32, [1, 2])
    assert np.abs(grid).max() > 2 ** 31, "the fixture must exercise int32 wrapping"


def test_fp64_oracle_tracks_reference_within_tolerance(oracle):
    g = golden("ref_head.npz")
    out, _ = run_snapshots(oracle, g, np.float64, [1, 10, 60])
    e1 = rel_pos_err(out[1], g["state_1"], N, REF_LENGTH)
    e60 = rel_pos_err(out[60], g["state_60"], N, REF_LENGTH)
    assert e1[0] <= 1e-5, e1
    # FP32 rounding alone, grown over 60 chaotic frames (penalty contacts + friction)
    assert e60[0] <= 5e-3 and e60[2] <= 1e-4, e60


def _hanging_strand(n, r, dftl):
    st = np.zeros((1, 3 * n, 4), np.float64)
    for j in range(n):
        st[0, j] = (0.0, -j * r, 0.0, 1.0)
    return st


def test_known_answer_hanging_strand_one_step(oracle):
    """Straight strand hanging under gravity, at rest, no colliders, no grid:
    FTL keeps every point; corr = dftl*(0, dt^2 g, 0); DFTL gives v_i = -dftl*dt*g_y*y for i < n-1."""
    n, r, dt, dftl, g = 8, float(np.float32(0.1)), 1.0 / 60.0, 0.9, 9.8
    P = T.reference_params()
    P.grid_enabled = 0
    P.dftl_damping = dftl
    st = _hanging_strand(n, r, dftl)
    x0 = st.copy()
    oracle.run(st, n, np.array([r], np.float32), P, T.frame(dt), [], 1)
    dtf = float(np.float32(dt))
    assert np.allclose(st[0, :n, :3], x0[0, :n, :3], atol=1e-15)
    corr = st[0, 2 * n:3 * n, :3]
    assert np.allclose(corr[1:], [0.0, float(np.float32(dftl)) * dtf * dtf * float(np.float32(g)), 0.0], rtol=1e-6)
    v = st[0, n:2 * n, :3]
    expect = -dftl * dtf * float(np.float32(g))
    assert np.allclose(v[1:n - 1, 1], expect, rtol=1e-6) and np.allclose(v[1:n - 1, [0, 2]], 0.0)
    assert np.allclose(v[n - 1], 0.0, atol=1e-15)
    assert np.array_equal(st[0, 0], x0[0, 0]) and np.array_equal(st[0, n], x0[0, n])


def test_known_answer_penalty_force(oracle):
    """Two-point strand whose tip starts inside a sphere: f = g + k d n, then FTL."""
    dt, k, R = 1.0 / 60.0, 1900.0, 0.5
    P = T.reference_params()
    P.grid_enabled = 0
    st = np.zeros((1, 6, 4), np.float64)
    st[0, 0] = (0.0, 0.0, 0.0, 1.0)
    st[0, 1] = (0.3, 0.0, 0.0, 1.0)
    centre = np.array([0.6, 0.1, 0.0])
    col = T.sphere_collider(centre, R)
    oracle.run(st, 2, np.array([0.3], np.float32), P, T.frame(dt), [col], 1)
    x = np.array([0.3, 0.0, 0.0])
    dtf = float(np.float32(dt))
    e = x - centre.astype(np.float32).astype(np.float64)
    d = float(np.float32(R)) - np.linalg.norm(e)
    f = np.array([0.0, float(np.float32(-9.8)), 0.0]) + float(np.float32(k)) * d * e / np.linalg.norm(e)
    pred = x + dtf * dtf * f
    newpos = float(np.float32(0.3)) * pred / np.linalg.norm(pred)
    assert np.allclose(st[0, 1, :3], newpos, rtol=0, atol=1e-12)


def test_invariants_root_pinned_segments_and_clamp(oracle):
    g = golden("ref_head.npz")
    out, _ = run_snapshots(oracle, g, np.float64, [1, 10])
    for s, st in out.items():
        assert np.array_equal(st[:, 0], g["init"][:, 0].astype(np.float64))       # root position
        assert np.array_equal(st[:, N], g["init"][:, N].astype(np.float64))       # root velocity
        seg = np.linalg.norm(np.diff(st[:, :N, :3], axis=1), axis=2)
        r = float(np.float32(2.5) / (np.float32(10) - np.float32(1.0)))
        assert np.abs(seg - r).max() / REF_LENGTH < 1e-12
        assert np.all(st[:, :N, 3] == 1.0) and np.all(st[:, N:, 3] == 0.0)
    # clamp: without DFTL and grid the stored velocity is the clamped one
    P = T.reference_params()
    P.grid_enabled = 0
    P.dftl_damping = 0.0
    frames, rows = ref_frames_and_colliders(g)
    st = g["init"].astype(np.float64)
    oracle.run(st, N, np.full(st.shape[0], 2.5 / 9.0, np.float32), P, frames[:1], rows[:1], 1)
    speed = np.linalg.norm(st[:, N:2 * N, :3], axis=2)
    assert speed.max() <= 10.0 * (1 + 1e-12) and speed.max() > 9.0


def test_splat_mass_conservation(oracle):
    """Each interior point splats total weight 1: sum(density) = SCALE * points, minus < 8 per point."""
    g = golden("ref_head.npz")
    frames, rows = ref_frames_and_colliders(g)
    st = g["init"].astype(np.float64)
    P = T.reference_params()
    P.grid_wrap32 = 0
    grid = oracle.run(st, N, np.full(st.shape[0], 2.5 / 9.0, np.float32), P, frames[:1], rows[:1], 1,
                      want_grid=True)
    gx = (st[:, 1:N, :3] - np.array([-3.0, -2.0, -5.0])) / (7.0 / 64.0)
    inside = np.all((gx >= 0) & (gx < 63), axis=2)
    total = grid[:, 3].sum()
    pts = st.shape[0] * (N - 1)
    n_in = int(inside.sum())
    assert n_in > 0.5 * pts
    # interior points contribute in [1e6 - 8, 1e6] each (8 truncations); boundary points less
    assert n_in * (1e6 - 8) <= total <= pts * 1e6


def test_oracle_threads_do_not_change_bits(oracle):
    from rvh import configs
    spec = configs.batched(n_assets=1, scale=0.05)[0]
    a = spec.records.astype(np.float64)
    b = a.copy()
    fr = [spec.frame(k) for k in range(3)]
    oracle.run(a, spec.n_points, spec.rest, spec.params, fr, spec.colliders, 3, threads=1)
    oracle.run(b, spec.n_points, spec.rest, spec.params, fr, spec.colliders, 3, threads=4)
    assert np.array_equal(a, b)
