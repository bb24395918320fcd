"""Assets sharing one hair-hair grid (the reference's one Scene grid for every
hair, src/Renderer.cpp:2063-2071, src/Scene.h:75-77).  The oracle's group step
(every member's loops 1-2 and splat before any member's loop 3) is checked
here on the CPU; the batched GPU path against it in the gpu tests."""
import numpy as np
import pytest

from rvh import api, configs
from rvh._lib import RvhError


def group_specs(n=3, seed=9, scale=0.01):
    specs = configs.batched(n_assets=n, seed=seed, scale=scale)
    g = specs[0].params
    for s in specs[1:]:   # one grid geometry for the group: the first member's
        p = s.params
        p.grid_dims[0], p.grid_dims[1], p.grid_dims[2] = g.grid_dims[0], g.grid_dims[1], g.grid_dims[2]
        p.grid_h, p.grid_scale, p.grid_wrap32 = g.grid_h, g.grid_scale, g.grid_wrap32
        p.grid_origin[0], p.grid_origin[1], p.grid_origin[2] = g.grid_origin[0], g.grid_origin[1], g.grid_origin[2]
    return specs


def test_oracle_group_of_one_is_the_asset_step(oracle):
    s = group_specs(1)[0]
    a = s.records.astype(np.float32).copy()
    b = s.records.astype(np.float32).copy()
    frames = [s.frame(k) for k in range(3)]
    oracle.run(a, s.n_points, s.rest, s.params, frames, s.colliders, 3)
    oracle.run_group([b], [s.n_points], [s.rest], [s.params], frames, s.colliders, 3)
    assert np.array_equal(a, b)


def test_oracle_group_couples_overlapping_assets(oracle):
    specs = group_specs(2)
    frames = [specs[0].frame(k) for k in range(3)]
    sep = [s.records.astype(np.float64).copy() for s in specs]
    for st, s in zip(sep, specs):
        oracle.run(st, s.n_points, s.rest, s.params, frames, specs[0].colliders, 3)
    grp = [s.records.astype(np.float64).copy() for s in specs]
    oracle.run_group(grp, [s.n_points for s in specs], [s.rest for s in specs], [s.params for s in specs], frames,
                     specs[0].colliders, 3)
    # the heads overlap, so each member's friction sees the other's strands
    for a, b in zip(sep, grp):
        assert np.isfinite(b).all()
        assert not np.array_equal(a, b)
    # positions still keep their segment lengths (the grid only changes velocities)
    for st, s in zip(grp, specs):
        p = st[:, :s.n_points, :3]
        seg = np.linalg.norm(np.diff(p, axis=1), axis=2)
        assert np.abs(seg - s.rest[:, None]).max() < 1e-6 * max(1.0, float(s.rest.max()))


def test_oracle_group_rejects_different_grid_geometry(oracle):
    specs = configs.batched(n_assets=2, seed=9, scale=0.01)
    assert list(specs[0].params.grid_dims) != list(specs[1].params.grid_dims)
    st = [s.records.astype(np.float32).copy() for s in specs]
    with pytest.raises(RuntimeError):
        oracle.run_group(st, [s.n_points for s in specs], [s.rest for s in specs], [s.params for s in specs],
                         [specs[0].frame(0)], specs[0].colliders, 1)


# ---- GPU: the batched path against the oracle's group step --------------------------------

def _assets(ctx, specs):
    out = []
    for s in specs:
        a = api.Asset(ctx, s.records, s.n_points, rest=s.rest)
        a.set_params(s.params)
        a.set_colliders(specs[0].colliders)   # the scene's colliders, shared
        out.append(a)
    return out


def _oracle_group(oracle, specs, steps):
    st = [s.records.astype(np.float32).copy() for s in specs]
    oracle.run_group(st, [s.n_points for s in specs], [s.rest for s in specs], [s.params for s in specs],
                     [specs[0].frame(k) for k in range(steps)], specs[0].colliders, steps)
    return st


@pytest.mark.gpu
@pytest.mark.parametrize("lanes", [8, 1])
def test_gpu_group_matches_the_oracle_group_step(gpu_ctx, oracle, lanes):
    specs = group_specs(3)
    assets = _assets(gpu_ctx, specs)
    assets[1].share_grid(assets[0])
    assets[2].share_grid(assets[0])
    b = api.Batch(gpu_ctx, assets, lanes=lanes)
    for k in range(4):
        b.step([specs[0].frame(k)] * 3)
    b.finish()
    got = [a.read() for a in assets]
    b.close()
    want = _oracle_group(oracle, specs, 4)
    for i in range(3):
        assert np.array_equal(got[i], want[i]), i
    for a in assets:
        a.close()


@pytest.mark.gpu
def test_gpu_group_reading_a_member_between_steps(gpu_ctx, oracle):
    """Reading one member applies its pending friction alone; the group's next step
    still gathers the others' from the same grid."""
    specs = group_specs(3, seed=10)
    assets = _assets(gpu_ctx, specs)
    assets[1].share_grid(assets[0])
    assets[2].share_grid(assets[0])
    b = api.Batch(gpu_ctx, assets)
    for k in range(2):
        b.step([specs[0].frame(k)] * 3)
    mid = assets[1].read()
    want2 = _oracle_group(oracle, specs, 2)
    assert np.array_equal(mid, want2[1])
    b.step([specs[0].frame(2)] * 3)
    b.finish()
    want3 = _oracle_group(oracle, specs, 3)
    for i, a in enumerate(assets):
        assert np.array_equal(a.read(), want3[i]), i
    b.close()
    for a in assets:
        a.close()


@pytest.mark.gpu
def test_gpu_group_beside_an_asset_with_its_own_grid(gpu_ctx, oracle):
    specs = group_specs(2, seed=11)
    solo_spec = configs.batched(n_assets=1, seed=12, scale=0.01)[0]
    assets = _assets(gpu_ctx, specs)
    assets[1].share_grid(assets[0])
    solo = api.Asset(gpu_ctx, solo_spec.records, solo_spec.n_points, rest=solo_spec.rest)
    solo.set_params(solo_spec.params)
    solo.set_colliders(solo_spec.colliders)
    b = api.Batch(gpu_ctx, [assets[0], solo, assets[1]])
    for k in range(3):
        b.step([specs[0].frame(k), solo_spec.frame(k), specs[0].frame(k)])
    b.finish()
    want = _oracle_group(oracle, specs, 3)
    assert np.array_equal(assets[0].read(), want[0]) and np.array_equal(assets[1].read(), want[1])
    ref = solo_spec.records.astype(np.float32).copy()
    oracle.run(ref, solo_spec.n_points, solo_spec.rest, solo_spec.params, [solo_spec.frame(k) for k in range(3)],
               solo_spec.colliders, 3)
    assert np.array_equal(solo.read(), ref)
    b.close()
    for a in assets + [solo]:
        a.close()


@pytest.mark.gpu
def test_gpu_group_rules(gpu_ctx):
    specs = group_specs(2, seed=13)
    other = configs.batched(n_assets=1, seed=14, scale=0.01)[0]
    assets = _assets(gpu_ctx, specs)
    owner, member = assets
    member.share_grid(owner)
    with pytest.raises(RvhError) as e:   # a member's plain step
        member.step(specs[0].frame(0))
    assert e.value.status == api.T.ERR_STATE
    with pytest.raises(RvhError):        # the group split across batches
        api.Batch(gpu_ctx, [member])
    with pytest.raises(RvhError) as e:   # full steps
        api.Batch(gpu_ctx, assets, full_steps=True)
    assert e.value.status == api.T.ERR_UNSUPPORTED
    p = specs[1].params
    p.grid_dims[0] = p.grid_dims[0] + 2
    with pytest.raises(RvhError) as e:   # a new grid geometry
        member.set_params(p)
    assert e.value.status == api.T.ERR_STATE
    p.grid_dims[0] = p.grid_dims[0] - 2
    with pytest.raises(RvhError):        # a different geometry cannot join
        x = api.Asset(gpu_ctx, other.records, other.n_points, rest=other.rest)
        x.set_params(other.params)
        try:
            x.share_grid(owner)
        finally:
            x.close()
    with pytest.raises(RvhError) as e:   # an owner leaves only after its members
        owner.share_grid(None)
    assert e.value.status == api.T.ERR_STATE
    srv = api.Server(gpu_ctx, max_active=2, scratch_budget_bytes=64 << 20)
    with pytest.raises(RvhError) as e:
        srv.add_character(member)
    assert e.value.status == api.T.ERR_UNSUPPORTED
    srv.close()
    # a member that leaves steps on its own again
    member.share_grid(None)
    member.step(specs[1].frame(0))
    member.share_grid(owner)
    # destroying the owner gives the member a grid of its own
    owner.close()
    member.step(specs[1].frame(1))
    assert np.isfinite(member.read()).all()
    member.close()
