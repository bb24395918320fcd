"""GPU parity of the plain per-asset step (C ABI) against the oracle and the
reference shader's golden outputs.

Tolerances (FP32 positions vs the FP64 oracle, relative to strand length L):
  1 step: 1e-5; segment lengths: 1e-6 * L.  The 120-step bounds are in
  tests/test_gpu_error120.py.
Exact math mode: bit-identical to the oracle's FP32 twin, which is itself
bit-identical to the reference shader (tests/test_oracle_golden.py)."""
import numpy as np
import pytest

from conftest import golden, rel_pos_err
from rvh import api, configs
from rvh import types as T
from rvh._lib import RvhError

pytestmark = pytest.mark.gpu


def asset_from_spec(ctx, spec, lanes=0, records=None):
    a = api.Asset(ctx, spec.records if records is None else records, spec.n_points, rest=spec.rest,
                  strand_wind=spec.strand_wind, lanes=lanes)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders_at(0))
    return a


def gpu_run(a, spec, steps, start=0):
    for k in range(start, start + steps):
        a.set_colliders(spec.colliders_at(k))
        a.step(spec.frame(k))
    return a.read()


def oracle_run(oracle, spec, steps, dtype, start=0, threads=8, state=None):
    st = (spec.records if state is None else state).astype(dtype).copy()
    frames = [spec.frame(k) for k in range(start, start + steps)]
    rows = [spec.colliders_at(k) for k in range(start, start + steps)]
    grid = oracle.run(st, spec.n_points, spec.rest, spec.params, frames, rows, steps,
                      strand_wind=spec.strand_wind, threads=threads, want_grid=True)
    return st, grid


def strand_lengths(spec):
    return spec.rest.astype(np.float64) * (spec.n_points - 1)


def small_head(n_points, seed=3, n_strands=300, grid_res=24, repulsion=0.02):
    rec, rest, p, cols = api.generate_head(seed=seed, n_strands=n_strands, n_points=n_points, root_sampling=0,
                                           sort_roots=1, length_min=0.3, length_max=0.9, head_collider=1,
                                           n_ellipsoids=3, axis_min=0.2, axis_max=0.5, grid_res=grid_res,
                                           friction=0.05, repulsion=repulsion, dftl_damping=0.9)
    wind = api.WindDesc()
    wind.amplitude, wind.omega, wind.gust_sigma, wind.seed = 2.0, 0.5, 0.5, seed
    wind.dir[:] = (1.0, 0.0, 0.0)
    return configs.AssetSpec(rec, rest, p, cols, n_points, wind=wind)


# ---- the reference's own shader outputs ----------------------------------------

@pytest.mark.parametrize("case,snaps", [("ref_head.npz", [1, 10, 60]), ("ref_dense.npz", [1, 2])])
def test_reference_shader_golden_bit_exact(gpu_ctx, case, snaps):
    g = golden(case)
    n = int(g["n_points"])
    a = api.Asset(gpu_ctx, g["init"], n, uniform_rest=float(np.float32(2.5) / np.float32(9.0)))
    a.set_params(api.reference_params())
    cs, times = g["colliders"], g["times"]
    done = 0
    for s in snaps:
        for k in range(done, s):
            a.set_colliders([T.collider_from_flat48(cs[k, j], T.COLLIDER_SPHERE if j == 0 else T.COLLIDER_ELLIPSOID)
                             for j in range(cs.shape[1])])
            a.step(T.frame(times[k, 0], times[k, 1]))
        done = s
        got = a.read()
        assert np.array_equal(got, g["state_%d" % s]), "step %d: max diff %g" % (s, np.abs(got - g["state_%d" % s]).max())
    grid = a.read_grid(64 ** 3)
    dense = np.zeros((64 ** 3, 4), np.int32)
    dense[g["grid_index"]] = g["grid_value"]
    assert np.array_equal(grid.astype(np.uint64).astype(np.uint32).view(np.int32), dense)
    a.close()


# ---- exact mode == the FP32 twin for every compiled shape -----------------------

SHAPES = [(2, 1), (2, 4), (8, 1), (8, 2), (8, 4), (8, 8), (10, 1), (10, 2), (10, 4), (12, 4), (12, 8),
          (16, 2), (16, 4), (16, 8), (16, 16), (24, 4), (24, 8), (32, 4), (32, 8), (32, 16), (32, 32)]


@pytest.mark.parametrize("n,lanes", SHAPES)
def test_exact_equals_fp32_twin(gpu_ctx, oracle, n, lanes):
    from rvh._lib import load
    spec = small_head(n)
    try:
        a = asset_from_spec(gpu_ctx, spec, lanes=lanes)
    except RvhError as e:
        assert e.status == T.ERR_UNSUPPORTED
        pytest.skip("shape not compiled")
    got = gpu_run(a, spec, 3)
    ref, grid = oracle_run(oracle, spec, 3, np.float32)
    assert np.array_equal(got, ref), "max diff %g" % np.abs(got - ref).max()
    d = spec.params.grid_dims
    assert np.array_equal(a.read_grid(d[0] * d[1] * d[2]), grid)
    a.close()


# ---- fast mode within the FP64 tolerances ----------------------------------------

@pytest.mark.parametrize("which", ["plain_small", "full_head_small", "small_head32"])
def test_fast_one_step_within_1e5(gpu_ctx_fast, oracle, which):
    spec = {"plain_small": lambda: configs.plain_small(),
            "full_head_small": lambda: configs.full_head(n_strands=8000),
            "small_head32": lambda: small_head(32)}[which]()
    a = asset_from_spec(gpu_ctx_fast, spec)
    got = gpu_run(a, spec, 1)
    ref, _ = oracle_run(oracle, spec, 1, np.float64)
    L = strand_lengths(spec)
    err = rel_pos_err(got, ref, spec.n_points, L)
    print(which, "1-step FP64 error max %.3g p99 %.3g mean %.3g" % err)
    assert err[0] <= 1e-5, err
    seg = np.linalg.norm(np.diff(got[:, :spec.n_points, :3].astype(np.float64), axis=1), axis=2)
    seg_err = np.abs(seg - spec.rest.astype(np.float64)[:, None]) / L[:, None]
    assert seg_err.max() <= 1e-6, seg_err.max()
    a.close()


# ---- behaviour of the drop-in boundary ---------------------------------------------

def test_draw_indirect_positions_and_root_untouched(gpu_ctx_fast):
    spec = small_head(16)
    a = asset_from_spec(gpu_ctx_fast, spec)
    got = gpu_run(a, spec, 2)
    assert np.array_equal(got[:, 0], spec.records[:, 0])
    assert np.array_equal(got[:, 16], spec.records[:, 16])
    assert a.read_draw() == (spec.n_strands, 1, 0, 0)
    assert np.array_equal(a.read_positions(), got[:, :16])
    a.close()


def test_deterministic_and_repeatable(gpu_ctx_fast):
    spec = small_head(24, n_strands=2000, grid_res=32)
    outs = []
    for _ in range(2):
        a = asset_from_spec(gpu_ctx_fast, spec)
        outs.append(gpu_run(a, spec, 5))
        a.close()
    assert np.array_equal(outs[0], outs[1])


def test_empty_and_single_strand(gpu_ctx_fast, oracle):
    spec = small_head(8, n_strands=1)
    a = asset_from_spec(gpu_ctx_fast, spec)
    got = gpu_run(a, spec, 3)
    ref, _ = oracle_run(oracle, spec, 3, np.float64)
    assert rel_pos_err(got, ref, 8, strand_lengths(spec))[0] < 1e-5
    a.close()
    e = api.Asset(gpu_ctx_fast, np.zeros((0, 24, 4), np.float32), 8, uniform_rest=0.1)
    e.set_params(spec.params)
    e.step(spec.frame(0))
    assert e.read().shape == (0, 24, 4)
    e.close()


def test_invalid_arguments_are_rejected(gpu_ctx_fast):
    spec = small_head(8, n_strands=4)
    with pytest.raises(RvhError) as ei:
        api.Asset(gpu_ctx_fast, np.zeros((4, 99, 4), np.float32), 33, uniform_rest=0.1)
    assert ei.value.status == T.ERR_INVALID_ARG
    a = asset_from_spec(gpu_ctx_fast, spec)
    for bad in (T.frame(0.0), T.frame(-1.0), T.frame(float("nan"))):
        with pytest.raises(RvhError) as ei:
            a.step(bad)
        assert ei.value.status == T.ERR_INVALID_ARG
    p = T.SimParams.from_buffer_copy(spec.params)
    p.grid_h = 0.0
    with pytest.raises(RvhError):
        a.set_params(p)
    with pytest.raises(RvhError):
        a.set_colliders([spec.colliders[0]] * 9)
    with pytest.raises(RvhError) as ei:
        api.Asset(gpu_ctx_fast, spec.records, 8, rest=spec.rest, lanes=3)
    assert ei.value.status == T.ERR_UNSUPPORTED
    a.close()


def test_hbm_budget_admission(librvh):
    spec = small_head(32, n_strands=2000, grid_res=64)
    ctx = api.Context(hbm_budget_bytes=4 << 20)
    with pytest.raises(RvhError) as ei:
        a = api.Asset(ctx, spec.records, 32, rest=spec.rest)
        a.set_params(spec.params)   # two 64^3 grids (16 MiB) exceed 4 MiB
    assert ei.value.status == T.ERR_BUDGET
    used, budget = ctx.memory()
    assert used <= budget
    ctx.close()


def test_borrowed_device_buffer_zero_copy(gpu_ctx_fast, oracle):
    import torch
    spec = small_head(16, n_strands=500)
    buf = torch.from_numpy(spec.records.copy()).cuda()
    a = api.Asset(gpu_ctx_fast, spec.n_strands, 16, rest=spec.rest, location=T.MEM_DEVICE_BORROWED,
                  device_ptr=buf.data_ptr())
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    b = asset_from_spec(gpu_ctx_fast, spec)
    for k in range(3):
        a.step(spec.frame(k))
        b.step(spec.frame(k))
    gpu_ctx_fast.synchronize()
    assert np.array_equal(buf.cpu().numpy(), b.read())
    a.close()
    b.close()


@pytest.mark.parametrize("n", [2, 3, 5, 7, 9, 11, 13, 31])
def test_default_lanes_cover_every_point_count(gpu_ctx, oracle, n):
    """An asset created without lanes_per_strand steps for any n in [2, 32]
    (point counts without a fixed-size kernel take the generic one)."""
    spec = small_head(n, seed=n, n_strands=64, grid_res=12)
    a = asset_from_spec(gpu_ctx, spec)
    got = gpu_run(a, spec, 2)
    twin, _ = oracle_run(oracle, spec, 2, np.float32)
    assert np.array_equal(got, twin)
