"""The autotuner and the group boxes a fused step leaves for the next one.

The tuner times batched trials of every (lanes, tile) shape on the caller's
assets and restores their records after each.  Trials of one lane count whose
groups are one round (32-point strands at 4 lanes) share a group-box layout,
so a trial must not start from the boxes the previous one stored for records
that have since been restored.  More generally a stored box only bounds the
records its step wrote: records rewritten in place through the device pointer
must give the same bits as a path that keeps no boxes."""
import numpy as np
import pytest

from rvh import api, configs

pytestmark = pytest.mark.gpu


def make(ctx, specs):
    out = []
    for s in specs:
        a = api.Asset(ctx, s.records, s.n_points, rest=s.rest)
        a.set_params(s.params)
        a.set_colliders(s.colliders)
        out.append(a)
    return out


@pytest.fixture(scope="module")
def specs():
    # every point count, among them 32-point assets (one-round groups at 4 lanes)
    return configs.batched(n_assets=8, scale=0.03, seed=14)


def test_tuner_restores_records_and_the_tuned_batch_matches_plain(gpu_ctx, specs):
    assets = make(gpu_ctx, specs)
    before = [a.read() for a in assets]
    frames0 = [s.frame(0) for s in specs]
    tr = api.tune(gpu_ctx, assets, frames0, steps=1)
    assert tr.n_tried == 20 and tr.lanes_per_strand in (1, 4, 8, 16, 32)
    for a, b in zip(assets, before):
        assert np.array_equal(a.read(), b)
    batch = api.Batch(gpu_ctx, assets, lanes=tr.lanes_per_strand, strands_per_tile=tr.strands_per_tile)
    for k in range(3):
        batch.step([s.frame(k) for s in specs])
    batch.finish()
    got = [a.read() for a in assets]
    batch.close()
    for a in assets:
        a.close()
    for i, s in enumerate(specs):
        p = make(gpu_ctx, [s])[0]
        for k in range(3):
            p.step(s.frame(k))
        assert np.array_equal(got[i], p.read()), i
        p.close()


def _rewritten_run(ctx, specs, lanes):
    """Two fused steps, every position moved by (0.05, -0.03, 0.02) in place
    through the borrowed device buffer (the friction of step 2 still pending),
    then a third step; the records after it."""
    import torch
    bufs, assets = [], []
    for s in specs:
        t = torch.from_numpy(np.ascontiguousarray(s.records, np.float32).reshape(-1)).cuda()
        bufs.append(t)
        a = api.Asset(ctx, len(s.rest), s.n_points, rest=s.rest, location=api.T.MEM_DEVICE_BORROWED,
                      device_ptr=t.data_ptr())
        a.set_params(s.params)
        a.set_colliders(s.colliders)
        assets.append(a)
    torch.cuda.synchronize()
    batch = api.Batch(ctx, assets, lanes=lanes)
    for k in range(2):
        batch.step([s.frame(k) for s in specs])
    ctx.synchronize()
    shift = torch.tensor([0.05, -0.03, 0.02, 0.0], device="cuda")
    for t, s in zip(bufs, specs):
        rec = t.view(-1, 3 * s.n_points, 4)
        rec[:, 1:s.n_points, :] += shift   # positions; the roots stay
    torch.cuda.synchronize()
    batch.step([s.frame(2) for s in specs])
    batch.finish()
    ctx.synchronize()
    out = [t.cpu().numpy().copy() for t in bufs]
    batch.close()
    for a in assets:
        a.close()
    return out


def test_records_rewritten_in_place_give_the_bits_of_a_path_without_stored_boxes(gpu_ctx, specs):
    boxes = _rewritten_run(gpu_ctx, specs, lanes=4)     # stored group boxes, now stale
    plain = _rewritten_run(gpu_ctx, specs, lanes=1)     # one thread per strand: no stored boxes
    for i, (a, b) in enumerate(zip(boxes, plain)):
        assert np.isfinite(a).all()
        assert np.array_equal(a, b), i
