"""The C-ABI library loads, exports every entry point include/*.h declares,
and its structs have the same layout in C and in the ctypes mirror.  CPU only
(no compute call needs a GPU here)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT
from rvh import api
from rvh import types as T

HEADERS = ["rvh.h", "rvh_scene.h", "rvh_types.h"]


def declared_functions():
    names = []
    for h in HEADERS:
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w]+\s*\**\s+(rvh_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(librvh):
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(librvh, n)]
    assert not missing, missing


def test_every_declared_symbol_has_a_prototype():
    from rvh._lib import PROTOTYPES
    have = {p[0] for p in PROTOTYPES}
    missing = [n for n in declared_functions() if n not in have]
    assert not missing, missing


LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include "rvh.h"
#include "rvh_scene.h"
#define S(t) printf(#t " %zu\n", sizeof(t));
#define O(t, f) printf(#t "." #f " %zu\n", offsetof(t, f));
int main(void) {
  S(rvh_collider) S(rvh_sim_params) S(rvh_frame) S(rvh_draw_indirect) S(rvh_context_desc)
  S(rvh_asset_desc) S(rvh_batch_desc) S(rvh_head_desc) S(rvh_wind_desc) S(rvh_orbit)
  S(rvh_tune_desc) S(rvh_tune_result) S(rvh_server_desc) S(rvh_request) S(rvh_request_result) S(rvh_server_stats)
  S(rvh_mesh_roots_desc) O(rvh_mesh_roots_desc, seed) O(rvh_mesh_roots_desc, normal_mode)
  S(rvh_tess_desc) O(rvh_tess_desc, tip_width)
  S(rvh_shade_desc) O(rvh_shade_desc, light_proj) O(rvh_shade_desc, map_height) O(rvh_shade_desc, map_mode)
  S(rvh_health) O(rvh_health, worst_strand)
  S(rvh_snapshot_header) O(rvh_snapshot_header, params) O(rvh_snapshot_header, colliders) O(rvh_snapshot_header, head)
  O(rvh_collider, kind) O(rvh_collider, radius) O(rvh_sim_params, grid_enabled) O(rvh_sim_params, grid_dims)
  O(rvh_frame, wind) O(rvh_asset_desc, strands) O(rvh_asset_desc, rest_lengths) O(rvh_asset_desc, lanes_per_strand)
  O(rvh_head_desc, grid_res) O(rvh_head_desc, dftl_damping) O(rvh_wind_desc, seed)
  return 0;
}
"""


def test_struct_layouts_match_ctypes():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(src, "w").write(LAYOUT_C)
        subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    c_vals = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    py = {
        "rvh_collider": T.Collider, "rvh_sim_params": T.SimParams, "rvh_frame": T.Frame,
        "rvh_draw_indirect": T.DrawIndirect, "rvh_context_desc": api.ContextDesc, "rvh_asset_desc": api.AssetDesc,
        "rvh_batch_desc": api.BatchDesc, "rvh_head_desc": api.HeadDesc, "rvh_wind_desc": api.WindDesc,
        "rvh_orbit": api.Orbit, "rvh_tune_desc": api.TuneDesc, "rvh_tune_result": api.TuneResult,
        "rvh_server_desc": api.ServerDesc, "rvh_request": api.Request, "rvh_request_result": api.RequestResult,
        "rvh_server_stats": api.ServerStats, "rvh_mesh_roots_desc": api.MeshRootsDesc,
        "rvh_tess_desc": api.TessDesc, "rvh_shade_desc": api.ShadeDesc, "rvh_snapshot_header": api.SnapshotHeader, "rvh_health": api.Health,
    }
    for name, cls in py.items():
        assert int(c_vals[name]) == C.sizeof(cls), name
    for key, val in c_vals.items():
        if "." in key:
            s, f = key.split(".")
            assert getattr(py[s], f).offset == int(val), key


def test_context_without_gpu_reports_no_device(librvh):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    d = api.ContextDesc(0, 0, 0)
    st = librvh.rvh_context_create(C.byref(d), C.byref(h))
    assert st == T.ERR_NO_DEVICE
    assert librvh.rvh_last_error()


def test_status_strings_and_version(librvh):
    assert librvh.rvh_abi_version() == 1
    for s in range(9):
        assert librvh.rvh_status_string(s)


def test_kernel_opt_in_is_recorded_per_device(tmp_path):
    """cudaFuncSetAttribute applies to the current device only: the record of
    opted-in kernels must key on (device, kernel), so a second device runs the
    opt-in again for a kernel the first already has.  Compiled alone (host C++)."""
    src = tmp_path / "optin.cpp"
    src.write_text(r'''
#include <cstdio>
#include "rvh_optin.hpp"
int main() {
    rvh::OptInRecord r;
    int calls = 0, k1 = 0, k2 = 0;
    auto ok = [&] { ++calls; return true; };
    auto bad = [&] { ++calls; return false; };
    bool a = r.ensure(0, &k1, ok), b = r.ensure(0, &k1, ok);   // once per (device, kernel)
    bool c = r.ensure(1, &k1, ok);                             // another device: again
    bool d = r.ensure(1, &k2, bad), e = r.ensure(1, &k2, ok);  // a failure is not recorded
    std::printf("%d %d %d %d %d %d %zu\n", a, b, c, d, e, calls, r.size());
    return 0;
}
''')
    exe = tmp_path / "optin"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "realtime-vulkan-hair_gb300", "csrc"), str(src),
                    "-o", str(exe), "-lpthread"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["1", "1", "1", "0", "1", "4", "3"], out
