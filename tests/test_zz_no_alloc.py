"""rvh_step_noalloc: the plain step for callers that cannot let the library
allocate device memory (the caller owns every buffer; the grid scratch is a
static device array).  Checked through the C ABI against rvh_step on an asset
with the same inputs, on two calls in a row (the second call must start from
a cleared grid, not the first call's sums), with the grid on and off, with a
per-strand wind and with an explicit lane count.  Tolerance: bit-identical,
since both run the same kernels; anything looser would hide a stale-scratch
bug.  Also: an empty step writes the draw record; unaligned buffers are
rejected before any launch.

This file sorts last so a run that stops at the first failure has already run
every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from rvh import api, configs
from rvh import types as T

pytestmark = pytest.mark.gpu


class NoallocDesc(C.Structure):
    _fields_ = [("strands", C.c_void_p), ("rest_lengths", C.c_void_p), ("strand_wind", C.c_void_p),
                ("draw_indirect", C.c_void_p), ("n_strands", C.c_int32), ("n_points", C.c_int32),
                ("lanes_per_strand", C.c_int32), ("math", C.c_int32), ("params", C.POINTER(T.SimParams)),
                ("colliders", C.POINTER(T.Collider)), ("n_colliders", C.c_int32), ("reserved", C.c_int32)]


CASES = {
    # name: (grid enabled, per-strand wind, lanes per strand)
    "grid": (True, False, 0),
    "no_grid": (False, False, 0),
    "strand_wind": (True, True, 0),
    "lanes4": (True, False, 4),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("math", [api.MATH_EXACT, api.MATH_FAST])
def test_noalloc_step_matches_rvh_step_twice(librvh, math, case):
    import torch
    grid, use_wind, lanes = CASES[case]
    spec = configs.full_head(n_strands=3000, n_points=16, grid_res=48)
    n = spec.n_points
    params = T.SimParams.from_buffer_copy(spec.params)
    params.grid_enabled = 1 if grid else 0
    wind = None
    if use_wind:
        wind = np.random.default_rng(5).normal(0.0, 0.5, size=(spec.n_strands, 3)).astype(np.float32)
    with api.Context(math=math) as ctx:
        a = api.Asset(ctx, spec.records, n, rest=spec.rest, strand_wind=wind, lanes=lanes)
        a.set_params(params)
        a.set_colliders(spec.colliders)
        recs = torch.from_numpy(spec.records.copy()).cuda()
        rest = torch.from_numpy(spec.rest.copy()).cuda()
        draw = torch.full((4,), 7, dtype=torch.int32, device="cuda")
        wind4 = None
        if use_wind:
            wind4 = torch.zeros((spec.n_strands, 4), dtype=torch.float32, device="cuda")
            wind4[:, :3] = torch.from_numpy(wind).cuda()
        cols = (T.Collider * len(spec.colliders))(*spec.colliders)
        d = NoallocDesc(recs.data_ptr(), rest.data_ptr(), None if wind4 is None else wind4.data_ptr(),
                        draw.data_ptr(), spec.n_strands, n, lanes, math, C.pointer(params), cols,
                        len(spec.colliders), 0)
        torch.cuda.synchronize()
        for k in range(2):
            f = spec.frame(k)
            a.step(f)
            st = librvh.rvh_step_noalloc(C.byref(d), C.byref(f), None)
            assert st == 0, librvh.rvh_last_error()
            torch.cuda.synchronize()
            ref = a.read()
            got = recs.cpu().numpy()
            assert np.array_equal(got, ref), "call %d: max diff %g" % (k, np.abs(got - ref).max())
        assert tuple(draw.cpu().numpy()) == (spec.n_strands, 1, 0, 0)
        a.close()


def test_noalloc_empty_step_writes_the_draw_record(librvh):
    import torch
    spec = configs.full_head(n_strands=64, n_points=8, grid_res=16)
    params = T.SimParams.from_buffer_copy(spec.params)
    draw = torch.full((4,), 7, dtype=torch.int32, device="cuda")
    d = NoallocDesc(None, None, None, draw.data_ptr(), 0, 8, 0, 0, C.pointer(params), None, 0, 0)
    f = spec.frame(0)
    assert librvh.rvh_step_noalloc(C.byref(d), C.byref(f), None) == 0, librvh.rvh_last_error()
    torch.cuda.synchronize()
    assert tuple(draw.cpu().numpy()) == (0, 1, 0, 0)


def test_noalloc_rejects_unaligned_buffers(librvh):
    spec = configs.full_head(n_strands=64, n_points=8, grid_res=16)
    params = T.SimParams.from_buffer_copy(spec.params)
    f = spec.frame(0)
    for strands, wind in ((4096 + 4, None), (4096, 4096 + 8)):   # never dereferenced: rejected first
        d = NoallocDesc(strands, 4096, wind, None, spec.n_strands, 8, 0, 0, C.pointer(params), None, 0, 0)
        assert librvh.rvh_step_noalloc(C.byref(d), C.byref(f), None) == T.ERR_INVALID_ARG
        assert b"16-byte aligned" in librvh.rvh_last_error()


def test_noalloc_rejects_grids_over_the_limit(librvh):
    spec = configs.full_head(n_strands=64, n_points=8, grid_res=65)
    params = T.SimParams.from_buffer_copy(spec.params)
    d = NoallocDesc(16, 16, None, None, spec.n_strands, 8, 0, 0, C.pointer(params), None, 0, 0)
    f = spec.frame(0)
    assert librvh.rvh_step_noalloc(C.byref(d), C.byref(f), None) == T.ERR_INVALID_ARG
    assert b"RVH_NOALLOC_MAX_GRID_CELLS" in librvh.rvh_last_error()
