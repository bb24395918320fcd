"""Checkpoint / resume (rvh_asset_snapshot, rvh_asset_restore) and failure
detection (rvh_asset_health).

A restored asset continues with the same bits as the original: plain steps
with a grid, colliders, per-strand wind and a moving head; and an asset whose
last step was a fused batched one (the snapshot finishes its pending friction).
Corrupt or truncated snapshots are rejected before anything is created.
"""
import numpy as np
import pytest

from rvh import api, configs

pytestmark = pytest.mark.gpu


def _head_asset(ctx, seed=4):
    rec, rest, p, cols = api.generate_head(seed=seed, n_strands=600, n_points=16, root_sampling=0, sort_roots=1,
                                           length_min=0.3, length_max=0.8, head_collider=1, n_ellipsoids=2,
                                           axis_min=0.2, axis_max=0.4, grid_res=32, friction=0.05, repulsion=0.02,
                                           dftl_damping=0.9)
    wind = np.random.default_rng(seed).normal(0.0, 0.3, (rec.shape[0], 3)).astype(np.float32)
    a = api.Asset(ctx, rec, 16, rest=rest, strand_wind=wind)
    a.set_params(p)
    for c in cols:
        c.attach_to_head = 1
    a.set_colliders(cols)
    return a


def _pose(k):
    t = 0.02 * k
    m = np.eye(4, dtype=np.float32)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = np.cos(t), np.sin(t), -np.sin(t), np.cos(t)
    m[1, 3] = 0.01 * k
    return m


def _frame(k):
    return api.T.frame(np.float32(1.0 / 60.0), np.float32((k + 1) / 60.0))


@pytest.mark.parametrize("ctx_name", ["gpu_ctx", "gpu_ctx_fast"])
def test_restored_asset_continues_bit_for_bit(request, ctx_name):
    ctx = request.getfixturevalue(ctx_name)
    a = _head_asset(ctx)
    for k in range(4):
        a.set_head_transform(_pose(k))
        a.step(_frame(k))
    snap = a.snapshot()
    b = api.Asset.restore(ctx, snap)
    assert b.snapshot() == snap
    for k in range(4, 9):
        for x in (a, b):
            x.set_head_transform(_pose(k))
            x.step(_frame(k))
    assert np.array_equal(a.read(), b.read())
    assert a.snapshot() == b.snapshot()
    a.close()
    b.close()


def test_restore_after_fused_batched_steps(gpu_ctx_fast):
    specs = configs.batched(n_assets=3, scale=0.02, seed=41)

    def make(s):
        x = api.Asset(gpu_ctx_fast, s.records, s.n_points, rest=s.rest, strand_wind=s.strand_wind)
        x.set_params(s.params)
        x.set_colliders(s.colliders)
        return x

    plain = [make(s) for s in specs]
    batched = [make(s) for s in specs]
    b = api.Batch(gpu_ctx_fast, batched, lanes=8)
    for k in range(3):
        b.step([s.frame(k) for s in specs])
        for x, s in zip(plain, specs):
            x.step(s.frame(k))
    restored = [api.Asset.restore(gpu_ctx_fast, x.snapshot()) for x in batched]   # finishes the pending friction
    for k in range(3, 6):
        for x, y, s in zip(plain, restored, specs):
            x.step(s.frame(k))
            y.step(s.frame(k))
    for x, y in zip(plain, restored):
        assert np.array_equal(x.read(), y.read())
    b.close()
    for x in plain + batched + restored:
        x.close()


def test_corrupt_snapshots_are_rejected(gpu_ctx):
    from rvh._lib import RvhError
    a = _head_asset(gpu_ctx, seed=5)
    a.set_head_transform(_pose(1))
    snap = bytearray(a.snapshot())
    a.close()
    bad_magic = bytearray(snap)
    bad_magic[0] ^= 0xFF
    for data in (bytes(bad_magic), bytes(snap[:-16]), bytes(snap[:40])):
        with pytest.raises(RvhError):
            api.Asset.restore(gpu_ctx, data)
    h = api.SnapshotHeader.from_buffer_copy(bytes(snap[:api.C.sizeof(api.SnapshotHeader)]))
    assert h.magic == b"RVHSNAP" and h.version == 1 and h.n_points == 16
    assert h.flags == 7   # wind, rest roots, head active


def test_health_of_a_running_and_a_corrupted_asset(gpu_ctx_fast):
    """A stepped asset is healthy (finite, segments at rest length); NaN, Inf and a
    stretched segment written into its records are reported."""
    a = _head_asset(gpu_ctx_fast, seed=6)
    for k in range(5):
        a.step(_frame(k))
    h = a.health()
    assert h.nonfinite == 0 and 0 < h.max_speed < 1e3
    assert h.max_length_error <= 1e-6 and 0 <= h.worst_strand < a.n_strands
    rec = a.read()
    rec[7, 3, 0] = np.nan               # strand 7: a position component
    rec[11, 16 + 2, 1] = np.inf         # strand 11: a velocity component
    rec[42, 5, :3] += np.float32(0.5)    # strand 42: a stretched segment
    a.write(rec)
    h = a.health()
    assert h.nonfinite == 2
    assert h.worst_strand == 42 and h.max_length_error > 0.1
    a.close()
