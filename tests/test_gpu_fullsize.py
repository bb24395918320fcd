"""The full-size workloads, through size-independent properties.

The 100k-strand head (100,000 strands x 32 points, 64^3 grid, 4 ellipsoids,
wind with gusts) over the 600 steps it is specified for, and the 256-head
batched workload (74.2 M points).  An FP64 oracle run of those sizes does not
finish in seconds, so the checks are what holds at any size: one step against
the FP64 oracle (1e-5 of strand length), inextensibility (segment length =
rest length within 1e-6 of strand length), the root pinned, finite state,
bitwise repeatability, batch = per-asset plain steps (fast math: every
kernel inlines the same device functions without implicit contraction), and
the positions a batched step stages for the host = the records it stored.
"""
import numpy as np
import pytest

from conftest import rel_pos_err
from rvh import api, configs

pytestmark = pytest.mark.gpu


def _asset(ctx, spec):
    a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest, strand_wind=spec.strand_wind)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders_at(0))
    return a


def _check_invariants(state, spec):
    n = spec.n_points
    assert np.isfinite(state).all()
    assert np.array_equal(state[:, 0], spec.records[:, 0])          # root position never written
    L = spec.rest.astype(np.float64) * (n - 1)
    seg = np.linalg.norm(np.diff(state[:, :n, :3].astype(np.float64), axis=1), axis=2)
    err = np.abs(seg - spec.rest.astype(np.float64)[:, None]) / L[:, None]
    assert err.max() <= 1e-6, err.max()
    assert (state[:, :n, 3] == 1.0).all() and (state[:, n:, 3] == 0.0).all()


def test_full_head_one_step_vs_fp64(gpu_ctx_fast, oracle):
    spec = configs.full_head()
    a = _asset(gpu_ctx_fast, spec)
    a.step(spec.frame(0))
    got = a.read()
    ref = spec.records.astype(np.float64)
    oracle.run(ref, spec.n_points, spec.rest, spec.params, [spec.frame(0)], [spec.colliders_at(0)], 1,
               threads=oracle.max_threads())
    L = spec.rest.astype(np.float64) * (spec.n_points - 1)
    err = rel_pos_err(got, ref, spec.n_points, L)
    print("full head, 1 step vs FP64: max %.3g p99 %.3g mean %.3g" % err)
    assert err[0] <= 1e-5, err
    a.close()


def test_full_head_600_steps_invariants_and_repeatability(gpu_ctx_fast):
    spec = configs.full_head()
    runs = []
    for _ in range(2):
        a = _asset(gpu_ctx_fast, spec)
        for k in range(600):
            a.set_colliders(spec.colliders_at(k))
            a.step(spec.frame(k))
        runs.append(a.read())
        a.close()
    _check_invariants(runs[0], spec)
    assert np.array_equal(runs[0], runs[1])


def test_batched_workload_full_size(gpu_ctx_fast):
    specs = configs.batched(n_assets=256)
    assets = [_asset(gpu_ctx_fast, s) for s in specs]
    b = api.Batch(gpu_ctx_fast, assets, lanes=8)
    steps = 4
    pts = b.info()["points"]
    assert pts == 74171408
    host = api.PinnedBuffer(pts * 12)
    for k in range(steps - 1):
        b.step([s.frame(k) for s in specs])
    b.step_read_positions([s.frame(steps - 1) for s in specs], host.ptr, pts * 12)   # the step stages its xyz
    b.positions_wait()
    b.check()
    staged = host.array((pts, 3))
    at = 0
    for a, s in zip(assets, specs):
        cnt = s.n_strands * s.n_points
        assert np.array_equal(staged[at:at + cnt], a.read()[:, :s.n_points, :3].reshape(-1, 3))
        at += cnt
    host.close()
    picks = [0, 17, 128, 255]                   # plain steps of a few assets give the same bits
    for i in picks:
        s = specs[i]
        p = _asset(gpu_ctx_fast, s)
        for k in range(steps):
            p.step(s.frame(k))
        got = assets[i].read()
        assert np.array_equal(got, p.read()), i
        _check_invariants(got, s)
        p.close()
    for i in range(0, 256, 32):
        _check_invariants(assets[i].read(), specs[i])
    b.close()
    for a in assets:
        a.close()
