"""Position error after 120 steps against the FP64 oracle, on the plain
workload, the full 100k-strand head and a sample of the batched workload
(one asset per point count, each with its hair-hair grid, stepped through
the batched launch).

Bounds (error = |x - x_fp64| / L per curve point, L the strand length):
  * exact math equals the FP32 twin bit for bit after 120 steps (the twin
    equals the reference shader's own arithmetic, tests/test_oracle_golden.py);
  * plain workload (no grid): every point of every well-conditioned strand is
    within 1e-3 (oracle/errors.py: an FP32-sized perturbation of the initial
    state grows less than 1000x in FP64 over the 120 steps);
  * grid workloads: the FP32 twin itself (the reference's arithmetic) is far
    from FP64 on many strands, because int(scale * w * v) truncation in nearly
    empty cells and the penalty branch are discontinuous; there the fast path
    must be no less accurate than the twin: p99 and mean at most 2x the
    twin's, the share of points within 1e-3 at most 2 points below it; segment
    lengths stay within 1e-6 L.
Each test prints max / p99 / mean / share within 1e-3 for both.
"""
import numpy as np
import pytest

from oracle import errors as E
from rvh import api, configs

pytestmark = pytest.mark.gpu

STEPS = 120


def _asset(ctx, spec):
    a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest, strand_wind=spec.strand_wind)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders_at(0))
    return a


def _plain_steps(ctx, spec, steps):
    a = _asset(ctx, spec)
    for k in range(steps):
        a.set_colliders(spec.colliders_at(k))
        a.step(spec.frame(k))
    out = a.read()
    a.close()
    return out


def _fmt(s):
    return "max %.3g p99 %.3g mean %.3g within1e-3 %.4f" % (s["max"], s["p99"], s["mean"], s["within_1e-3"])


def _no_worse_than_twin(fast, twin):
    assert fast["p99"] <= 2.0 * twin["p99"] + 1e-6, (fast, twin)
    assert fast["mean"] <= 2.0 * twin["mean"] + 1e-7, (fast, twin)
    assert fast["within_1e-3"] >= twin["within_1e-3"] - 0.02, (fast, twin)


def test_plain_workload_well_conditioned_within_1e3(gpu_ctx, gpu_ctx_fast, oracle):
    spec = configs.plain_small()
    thr = oracle.max_threads()
    L = E.lengths(spec.rest, spec.n_points)
    ref = E.run_spec(spec, STEPS, np.float64, thr)
    twin = E.run_spec(spec, STEPS, np.float32, thr)
    well = E.spread(spec, STEPS, ref, thr, seeds=(1, 2, 3)) <= 1e-4
    assert well.mean() > 0.75, well.mean()
    for ctx, name in ((gpu_ctx, "exact"), (gpu_ctx_fast, "fast")):
        got = _plain_steps(ctx, spec, STEPS)
        e = E.point_errors(got, ref, spec.n_points, L)
        print(name, "120 steps: all", _fmt(E.summary(e)), "| well-conditioned (%d of %d strands)" % (
            well.sum(), spec.n_strands), _fmt(E.summary(e[well])))
        if name == "exact":
            assert np.array_equal(got, twin)
        assert e[well].max() <= 1e-3, E.summary(e[well])
        assert E.segment_error(got, spec.rest, spec.n_points) <= 1e-6


def test_full_head_120_steps(gpu_ctx, gpu_ctx_fast, oracle):
    spec = configs.full_head()
    thr = oracle.max_threads()
    L = E.lengths(spec.rest, spec.n_points)
    ref = E.run_spec(spec, STEPS, np.float64, thr)
    twin = E.run_spec(spec, STEPS, np.float32, thr)
    st = E.summary(E.point_errors(twin, ref, spec.n_points, L))
    print("full head, 120 steps: FP32 twin", _fmt(st))
    assert np.array_equal(_plain_steps(gpu_ctx, spec, STEPS), twin)
    got = _plain_steps(gpu_ctx_fast, spec, STEPS)
    sf = E.summary(E.point_errors(got, ref, spec.n_points, L))
    print("full head, 120 steps: fast      ", _fmt(sf))
    _no_worse_than_twin(sf, st)
    assert E.segment_error(got, spec.rest, spec.n_points) <= 1e-6


def _batched_sample():
    """The first asset of each point count in the batched workload's order."""
    picks = {}
    for i, (ns, n, res, ne) in enumerate(configs.batched_sizes(256)):
        picks.setdefault(n, i)
    return configs.batched(n_assets=256, indices=[picks[n] for n in sorted(picks)])


@pytest.mark.parametrize("lanes", [0, 1])
def test_batched_sample_120_steps(gpu_ctx, gpu_ctx_fast, oracle, lanes):
    specs = _batched_sample()
    assert sorted(s.n_points for s in specs) == [8, 16, 24, 32] and all(s.params.grid_enabled for s in specs)
    thr = oracle.max_threads()
    out = {}
    for ctx, name in ((gpu_ctx, "exact"), (gpu_ctx_fast, "fast")):
        assets = [_asset(ctx, s) for s in specs]
        b = api.Batch(ctx, assets, lanes=lanes)
        for k in range(STEPS):
            b.step([s.frame(k) for s in specs])
        b.finish()
        b.check()
        out[name] = [a.read() for a in assets]
        b.close()
        for a in assets:
            a.close()
    et, ef = [], []
    for i, s in enumerate(specs):
        L = E.lengths(s.rest, s.n_points)
        ref = E.run_spec(s, STEPS, np.float64, thr)
        twin = E.run_spec(s, STEPS, np.float32, thr)
        assert np.array_equal(out["exact"][i], twin), "asset with %d points" % s.n_points
        assert E.segment_error(out["fast"][i], s.rest, s.n_points) <= 1e-6
        et.append(E.point_errors(twin, ref, s.n_points, L).reshape(-1))
        ef.append(E.point_errors(out["fast"][i], ref, s.n_points, L).reshape(-1))
        print("asset %d strands x %d points: twin %s | fast %s" % (
            s.n_strands, s.n_points, _fmt(E.summary(et[-1])), _fmt(E.summary(ef[-1]))))
    _no_worse_than_twin(E.summary(np.concatenate(ef)), E.summary(np.concatenate(et)))
