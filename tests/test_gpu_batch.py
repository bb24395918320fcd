"""The batched persistent launch computes exactly what per-asset plain steps
compute (same device functions, per-asset grids, exact integer sums)."""
import numpy as np
import pytest

from conftest import rel_pos_err
from rvh import api, configs

pytestmark = pytest.mark.gpu


def make_assets(ctx, specs):
    out = []
    for s in specs:
        a = api.Asset(ctx, s.records, s.n_points, rest=s.rest, strand_wind=s.strand_wind)
        a.set_params(s.params)
        a.set_colliders(s.colliders_at(0))
        out.append(a)
    return out


@pytest.mark.parametrize("lanes", [4, 8, 16, 32])
@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_equals_plain(gpu_ctx_fast, lanes, use_graph):
    """Fast math: the register kernels share every device function with the
    plain step, so the bits agree (the one-thread-per-strand kernel contracts
    differently in fast math and is checked in exact math below)."""
    specs = configs.batched(n_assets=10, scale=0.03)
    plain = make_assets(gpu_ctx_fast, specs)
    batched = make_assets(gpu_ctx_fast, specs)
    b = api.Batch(gpu_ctx_fast, batched, lanes=lanes, use_graph=use_graph)
    for k in range(4):
        for a, s in zip(plain, specs):
            a.step(s.frame(k))
        b.step([s.frame(k) for s in specs])
    b.check()
    for a, c, s in zip(plain, batched, specs):
        x, y = a.read(), c.read()
        assert np.array_equal(x, y), "max diff %g" % np.abs(x - y).max()
        assert c.read_draw() == (s.n_strands, 1, 0, 0)
    info = b.info()
    assert info["points"] == sum(s.n_total_points for s in specs)
    b.close()
    for a in plain + batched:
        a.close()


@pytest.mark.parametrize("lanes", [0, 1])
def test_batch_exact_equals_fp32_twin(gpu_ctx, oracle, lanes):
    specs = configs.batched(n_assets=6, scale=0.02, seed=9)
    assets = make_assets(gpu_ctx, specs)
    b = api.Batch(gpu_ctx, assets, lanes=lanes)
    steps = 3
    for k in range(steps):
        b.step([s.frame(k) for s in specs])
    b.check()
    for a, s in zip(assets, specs):
        ref = s.records.copy()
        oracle.run(ref, s.n_points, s.rest, s.params, [s.frame(k) for k in range(steps)], s.colliders, steps,
                   threads=8)
        assert np.array_equal(a.read(), ref)
        ref64 = s.records.astype(np.float64)
        oracle.run(ref64, s.n_points, s.rest, s.params, [s.frame(k) for k in range(steps)], s.colliders, steps,
                   threads=8)
        err = rel_pos_err(a.read(), ref64, s.n_points, s.rest.astype(np.float64) * (s.n_points - 1))
        # the max is set by fixed-point quantisation in nearly empty grid cells (int(1e6*w*v)
        # with 1e6*w ~ 1 truncates differently in FP32 and FP64); p99 and mean are rounding-level
        assert err[1] < 1e-5 and err[2] < 1e-6, err
    b.close()
    for a in assets:
        a.close()


def test_batch_then_plain_then_batch(gpu_ctx_fast):
    """Mixing the two paths on one asset keeps each grid clean before use."""
    specs = configs.batched(n_assets=4, scale=0.02, seed=11)
    x = make_assets(gpu_ctx_fast, specs)
    y = make_assets(gpu_ctx_fast, specs)
    b = api.Batch(gpu_ctx_fast, x)
    for k in range(5):
        if k == 2:
            for a, s in zip(x, specs):
                a.step(s.frame(k))
        else:
            b.step([s.frame(k) for s in specs])
        for a, s in zip(y, specs):
            a.step(s.frame(k))
    b.check()
    for a, c in zip(x, y):
        assert np.array_equal(a.read(), c.read())
    b.close()
    for a in x + y:
        a.close()


@pytest.mark.parametrize("steps", [1, 5])
def test_streaming_kernel_exact_equals_plain(gpu_ctx, steps):
    """lanes_per_strand = 1 (one thread walks each strand) in exact math: the
    same bits as the plain step, over fused steps and with a pending finish."""
    specs = configs.batched(n_assets=8, scale=0.03, seed=5)
    plain = make_assets(gpu_ctx, specs)
    batched = make_assets(gpu_ctx, specs)
    b = api.Batch(gpu_ctx, batched, lanes=1)
    for k in range(steps):
        for a, s in zip(plain, specs):
            a.step(s.frame(k))
        b.step([s.frame(k) for s in specs])
    b.check()
    for a, c in zip(plain, batched):
        x, y = a.read(), c.read()
        assert np.array_equal(x, y), "max diff %g" % np.abs(x - y).max()
    b.close()


def test_streaming_kernel_fast_close_to_fp64(gpu_ctx_fast, oracle):
    specs = configs.batched(n_assets=4, scale=0.02, seed=6)
    assets = make_assets(gpu_ctx_fast, specs)
    b = api.Batch(gpu_ctx_fast, assets, lanes=1)
    b.step([s.frame(0) for s in specs])
    for a, s in zip(assets, specs):
        ref64 = s.records.astype(np.float64)
        oracle.run(ref64, s.n_points, s.rest, s.params, [s.frame(0)], s.colliders, 1, threads=8)
        L = s.rest.astype(np.float64) * (s.n_points - 1)
        mx, p99, mean = rel_pos_err(a.read(), ref64, s.n_points, L)
        assert mx <= 1e-5, (mx, p99, mean)
    b.close()


@pytest.mark.parametrize("xyz", [False, True])
def test_batch_positions_read_back(gpu_ctx_fast, xyz):
    """rvh_batch_read_positions_async: every asset's curvePoints in batch order,
    as float4 records or as xyz triples, equal to the assets' own reads."""
    specs = configs.batched(n_assets=5, scale=0.02, seed=21)
    assets = make_assets(gpu_ctx_fast, specs)
    b = api.Batch(gpu_ctx_fast, assets, lanes=8)
    pts = b.info()["points"]
    width = 3 if xyz else 4
    bufs = [api.PinnedBuffer(pts * 4 * width) for _ in range(2)]
    for k in range(3):
        b.step([s.frame(k) for s in specs])
        b.read_positions_async(bufs[k % 2].ptr, pts * 4 * width)
    b.positions_wait()
    got = bufs[0].array((pts, width)).copy()   # the last step went to slot 0
    want = np.concatenate([a.read()[:, :s.n_points, :width].reshape(-1, width) for a, s in zip(assets, specs)])
    assert np.array_equal(got, want)
    for p_ in bufs:
        p_.close()
    b.close()


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("lanes", [1, 4, 8, 16, 32])
@pytest.mark.parametrize("pinned", [True, False])
def test_step_read_positions(gpu_ctx, gpu_ctx_fast, exact, lanes, pinned):
    """rvh_batch_step_read_positions: the step kernel's own xyz copy of every
    point (a moving head's roots included) equals the assets' reads, and the
    records equal those of a twin batch stepped without the copy, into page-locked
    and into pageable host memory."""
    ctx = gpu_ctx if exact else gpu_ctx_fast
    specs = configs.batched(n_assets=4, scale=0.02, seed=23)
    twin = make_assets(ctx, specs)
    assets = make_assets(ctx, specs)
    pose = np.eye(4, dtype=np.float32)
    pose[0, 3], pose[1, 3] = 0.05, -0.02
    for a in (twin[1], assets[1]):
        a.set_head_transform(pose)
    b = api.Batch(ctx, assets, lanes=lanes)
    bt = api.Batch(ctx, twin, lanes=lanes)
    pts = b.info()["points"]
    if pinned:
        bufs = [api.PinnedBuffer(pts * 12) for _ in range(2)]
        ptrs = [p_.ptr for p_ in bufs]
    else:
        pageable = [np.zeros((pts, 3), np.float32) for _ in range(2)]
        ptrs = [a_.ctypes.data for a_ in pageable]
    for k in range(3):
        b.step_read_positions([s.frame(k) for s in specs], ptrs[k % 2], pts * 12)
        bt.step([s.frame(k) for s in specs])
    b.positions_wait()
    got = (bufs[0].array((pts, 3)) if pinned else pageable[0]).copy()   # the last step went to buffer 0
    want = np.concatenate([a.read()[:, :s.n_points, :3].reshape(-1, 3) for a, s in zip(assets, specs)])
    assert np.array_equal(got, want)
    for a, t in zip(assets, twin):
        assert np.array_equal(a.read(), t.read())
    from rvh._lib import RvhError
    with pytest.raises(RvhError):
        b.step_read_positions([s.frame(3) for s in specs], ptrs[0], pts * 16)   # xyz only
    if pinned:
        for p_ in bufs:
            p_.close()
    b.close()
    bt.close()


class _DeviceArray:
    """A view of device memory through __cuda_array_interface__ (no copy)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (ptr, False), "version": 3}


def _raw_records(asset):
    """The asset's device records as they are: no finish on the way (rvh_asset_device_ptr)."""
    import torch
    torch.cuda.synchronize()
    n = asset.n_strands * 3 * asset.n_points * 4
    t = torch.as_tensor(_DeviceArray(asset.device_ptr(), n), device="cuda")
    return t.cpu().numpy().reshape(asset.n_strands, 3 * asset.n_points, 4)


@pytest.mark.parametrize("exact", [True, False])
def test_batched_finish_equals_plain(gpu_ctx, gpu_ctx_fast, exact):
    """rvh_batch_finish applies every asset's pending friction in one launch:
    right after it the device records (read raw, without the finish a read
    does) equal plain steps bit for bit; more fused steps after it, and a
    second finish, keep that."""
    ctx = gpu_ctx if exact else gpu_ctx_fast
    specs = configs.batched(n_assets=9, scale=0.03, seed=31)
    plain = make_assets(ctx, specs)
    batched = make_assets(ctx, specs)
    b = api.Batch(ctx, batched, lanes=8)

    def advance(k0, k1):
        for k in range(k0, k1):
            for a, s in zip(plain, specs):
                a.step(s.frame(k))
            b.step([s.frame(k) for s in specs])

    advance(0, 3)
    ctx.synchronize()
    before = [_raw_records(c) for c in batched]
    b.finish()
    b.check()
    changed = 0
    for a, c, old in zip(plain, batched, before):
        got = _raw_records(c)
        assert np.array_equal(a.read(), got)
        changed += not np.array_equal(old, got)
    assert changed > 0          # the pending friction was applied by the batched finish
    b.finish()                  # nothing pending: no change
    advance(3, 5)
    b.finish()
    b.check()
    for a, c in zip(plain, batched):
        assert np.array_equal(a.read(), _raw_records(c))
    b.close()
    for a in plain + batched:
        a.close()


def test_alternating_batch_groupings_equal_plain(gpu_ctx_fast):
    """A fused step reuses the cell boxes the previous fused step left for its
    phase-A groups only when both used the same grouping.  Fused steps of the
    same assets alternate here between batches with different lane counts (so
    different group boundaries); the result equals plain steps bit for bit."""
    specs = configs.batched(n_assets=6, scale=0.05, seed=11)
    plain = make_assets(gpu_ctx_fast, specs)
    shared = make_assets(gpu_ctx_fast, specs)
    batches = {lanes: api.Batch(gpu_ctx_fast, shared, lanes=lanes) for lanes in (4, 8, 16)}
    order = [8, 8, 16, 16, 8, 4, 8, 8]
    for k, lanes in enumerate(order):
        for a, s in zip(plain, specs):
            a.step(s.frame(k))
        batches[lanes].step([s.frame(k) for s in specs])
    for b in batches.values():
        b.check()
    for a, c in zip(plain, shared):
        x, y = a.read(), c.read()
        assert np.array_equal(x, y), "max diff %g" % np.abs(x - y).max()
    for b in batches.values():
        b.close()
    for a in plain + shared:
        a.close()
