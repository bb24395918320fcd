"""Serving: continuous batching of step requests for resident characters.
Each character's result is bit-identical whether its request runs alone or
shares launches with other requests (per-character grids, exact integer
sums, same frames), and admission respects slots and the HBM budget."""
import numpy as np
import pytest

from rvh import api, configs
from rvh import types as T
from rvh._lib import RvhError

pytestmark = pytest.mark.gpu


def characters(ctx, specs):
    out = []
    for s in specs:
        a = api.Asset(ctx, s.records, s.n_points, rest=s.rest)
        a.set_params(s.params)
        a.set_colliders(s.colliders)
        out.append(a)
    return out


def plain_reference(ctx, spec, steps):
    a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    for k in range(steps):
        a.step(spec.frame(k))
    out = a.read()
    a.close()
    return out


@pytest.fixture(scope="module")
def specs():
    return configs.batched(n_assets=6, scale=0.01, seed=21)


@pytest.mark.parametrize("spl", [1, 3, 8])   # steps of a request per launch
def test_served_result_is_the_same_alone_and_in_the_mix(gpu_ctx_fast, specs, spl):
    steps = [5, 3, 7, 2, 6, 4]
    # alone: one request for character 0
    srv = api.Server(gpu_ctx_fast, max_active=16, scratch_budget_bytes=256 << 20, steps_per_launch=spl)
    assets = characters(gpu_ctx_fast, specs)
    ids = [srv.add_character(a, wind=s.wind) for a, s in zip(assets, specs)]
    st, res, stats = srv.run([(ids[0], steps[0], 0.0)])
    assert st == 0 and res[0].status == 0 and res[0].steps_done == steps[0]
    alone = assets[0].read()
    srv.close()
    for a in assets:
        a.close()
    # in the mix: all six characters, arrivals spread over a few milliseconds
    srv = api.Server(gpu_ctx_fast, max_active=16, scratch_budget_bytes=256 << 20, steps_per_launch=spl)
    assets = characters(gpu_ctx_fast, specs)
    ids = [srv.add_character(a, wind=s.wind) for a, s in zip(assets, specs)]
    reqs = [(ids[i], steps[i], 0.002 * (i % 3)) for i in range(6)]
    st, res, stats = srv.run(reqs)
    assert st == 0 and all(r.status == 0 for r in res)
    assert [r.steps_done for r in res] == steps
    assert stats.mean_batch > 1.0, "requests should have shared launches"
    mixed = [a.read() for a in assets]
    assert np.array_equal(mixed[0], alone)
    for i, s in enumerate(specs):
        assert np.array_equal(mixed[i], plain_reference(gpu_ctx_fast, s, steps[i])), i
    assert stats.scratch_used_bytes == 0
    print({k: v for k, v in stats.as_dict().items()})
    srv.close()
    for a in assets:
        a.close()


@pytest.mark.parametrize("spl", [1, 2])
def test_consecutive_requests_for_one_character_continue_its_state(gpu_ctx_fast, specs, spl):
    srv = api.Server(gpu_ctx_fast, max_active=4, scratch_budget_bytes=256 << 20, steps_per_launch=spl)
    assets = characters(gpu_ctx_fast, specs[:2])
    ids = [srv.add_character(a, wind=s.wind) for a, s in zip(assets, specs[:2])]
    st, res, _ = srv.run([(ids[0], 2, 0.0), (ids[0], 3, 0.0), (ids[1], 4, 0.0)])
    assert st == 0 and all(r.status == 0 for r in res)
    assert srv.character_steps(ids[0]) == 5
    assert np.array_equal(assets[0].read(), plain_reference(gpu_ctx_fast, specs[0], 5))
    srv.close()
    for a in assets:
        a.close()


@pytest.mark.parametrize("spl", [1, 2])
def test_admission_respects_the_hbm_budget(gpu_ctx_fast, specs, spl):
    grid_pair = [2 * 32 * int(np.prod(list(s.params.grid_dims))) for s in specs]
    budget = 2 * max(grid_pair) + 4096
    srv = api.Server(gpu_ctx_fast, max_active=16, scratch_budget_bytes=budget, steps_per_launch=spl)
    assets = characters(gpu_ctx_fast, specs)
    ids = [srv.add_character(a, wind=s.wind) for a, s in zip(assets, specs)]
    st, res, stats = srv.run([(i, 3, 0.0) for i in ids])
    assert st == 0 and all(r.status == 0 and r.steps_done == 3 for r in res)
    # the two largest grid pairs fit at once, all six do not: admission had to wait
    assert stats.max_active < len(specs) and stats.admission_waits > 0
    for i, s in enumerate(specs):
        assert np.array_equal(assets[i].read(), plain_reference(gpu_ctx_fast, s, 3))
    srv.close()
    for a in assets:
        a.close()


@pytest.mark.parametrize("spl", [1, 3])
def test_characters_give_back_their_grids_when_space_is_short(gpu_ctx_fast, specs, spl):
    """Room for one character's grids: the characters take turns, and before the
    other is admitted the idle one's pending friction is applied and its grids freed."""
    sub = [specs[0], specs[1]]
    grids = [3 * ((32 * int(np.prod(list(s.params.grid_dims))) + 255) // 256 * 256) for s in sub]
    srv = api.Server(gpu_ctx_fast, max_active=4, scratch_budget_bytes=max(grids) + 4096, steps_per_launch=spl)
    assets = characters(gpu_ctx_fast, sub)
    ids = [srv.add_character(a, wind=s.wind) for a, s in zip(assets, sub)]
    st, res, stats = srv.run([(ids[0], 2, 0.0), (ids[1], 2, 0.0), (ids[0], 3, 0.0)])
    assert st == 0 and all(r.status == 0 for r in res)
    assert stats.max_active == 1 and stats.admission_waits > 0 and stats.scratch_used_bytes == 0
    assert np.array_equal(assets[0].read(), plain_reference(gpu_ctx_fast, sub[0], 5))
    assert np.array_equal(assets[1].read(), plain_reference(gpu_ctx_fast, sub[1], 2))
    srv.close()
    for a in assets:
        a.close()


def test_bad_requests_fail_alone(gpu_ctx_fast, specs):
    for bad in (-1, 17):   # steps per launch: 0 means 1, at most 16
        with pytest.raises(RvhError):
            api.Server(gpu_ctx_fast, max_active=4, scratch_budget_bytes=256 << 20, steps_per_launch=bad)
    srv = api.Server(gpu_ctx_fast, max_active=4, scratch_budget_bytes=256 << 20)
    assets = characters(gpu_ctx_fast, specs[:1])
    cid = srv.add_character(assets[0], wind=specs[0].wind)
    st, res, _ = srv.run([(cid, 2, 0.0), (99, 2, 0.0), (cid, 0, 0.0)])
    assert res[0].status == 0 and res[0].steps_done == 2
    assert res[1].status == T.ERR_INVALID_ARG and res[2].status == T.ERR_INVALID_ARG
    srv.close()
    assets[0].close()


@pytest.mark.parametrize("spl", [1, 4])
def test_poisson_trace_reports_latency(gpu_ctx_fast, spl):
    specs = configs.batched(n_assets=24, scale=0.05, seed=31)
    srv = api.Server(gpu_ctx_fast, max_active=8, scratch_budget_bytes=1 << 30, steps_per_launch=spl)
    assets = characters(gpu_ctx_fast, specs)
    ids = [srv.add_character(a, wind=s.wind) for a, s in zip(assets, specs)]
    rng = np.random.default_rng(5)
    t = np.cumsum(rng.exponential(1.0 / 5000.0, size=200))
    reqs = [(ids[int(rng.integers(0, len(ids)))], int(rng.integers(1, 9)), float(ti)) for ti in t]
    st, res, stats = srv.run(reqs)
    assert st == 0 and all(r.status == 0 for r in res)
    assert stats.steps == sum(k for _, k, _ in reqs)
    assert 0 < stats.step_ms_p50 <= stats.step_ms_p99 <= stats.step_ms_p999
    assert stats.point_steps_per_s > 0 and stats.max_active <= 8
    print({k: v for k, v in stats.as_dict().items()})
    srv.close()
    for a in assets:
        a.close()
