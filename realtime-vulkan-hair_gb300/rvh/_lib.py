"""ctypes bindings of include/rvh.h and include/rvh_scene.h.

The shared library is built in-tree (realtime-vulkan-hair_gb300/build.py ->
rvh/_build/librvh.so).  There is no fallback: if it is missing, load()
raises, so nothing silently runs without the CUDA kernels.
"""
import ctypes as C
import os

from . import types as T

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "librvh.so")

_P = C.POINTER
_vp = C.c_void_p
_st = C.c_int32

# (name, restype, argtypes) of every exported entry point
PROTOTYPES = [
    ("rvh_abi_version", C.c_int32, []),
    ("rvh_last_error", C.c_char_p, []),
    ("rvh_status_string", C.c_char_p, [_st]),
    ("rvh_context_create", _st, [_vp, _P(_vp)]),
    ("rvh_context_destroy", _st, [_vp]),
    ("rvh_context_synchronize", _st, [_vp]),
    ("rvh_pinned_alloc", _st, [C.c_size_t, _P(_vp)]),
    ("rvh_pinned_free", _st, [_vp]),
    ("rvh_context_memory", _st, [_vp, _P(C.c_uint64), _P(C.c_uint64)]),
    ("rvh_sim_params_reference", _st, [_P(T.SimParams)]),
    ("rvh_collider_from_trs", _st, [_P(C.c_float), _P(C.c_float), _P(C.c_float), C.c_int32, C.c_float,
                                    _P(T.Collider)]),
    ("rvh_collider_translate", _st, [_P(T.Collider), _P(C.c_float)]),
    ("rvh_collider_follow", _st, [_P(T.Collider), _P(C.c_float), _P(T.Collider)]),
    ("rvh_init_strands_reference", _st, [_P(C.c_float), _P(C.c_float), C.c_int32, C.c_int32, C.c_float,
                                         _P(C.c_float), _vp]),
    ("rvh_asset_create", _st, [_vp, _vp, _P(_vp)]),
    ("rvh_asset_destroy", _st, [_vp]),
    ("rvh_asset_set_params", _st, [_vp, _P(T.SimParams)]),
    ("rvh_asset_set_colliders", _st, [_vp, _P(T.Collider), C.c_int32]),
    ("rvh_asset_share_grid", _st, [_vp, _vp]),
    ("rvh_asset_set_head_transform", _st, [_vp, _P(C.c_float)]),
    ("rvh_asset_set_rest_lengths", _st, [_vp, _P(C.c_float)]),
    ("rvh_asset_set_strand_wind", _st, [_vp, _P(C.c_float)]),
    ("rvh_asset_device_ptr", _st, [_vp, _P(_vp)]),
    ("rvh_asset_draw_indirect", _st, [_vp, _P(_vp)]),
    ("rvh_asset_strand_count", _st, [_vp, _P(C.c_int32), _P(C.c_int32)]),
    ("rvh_asset_read", _st, [_vp, _vp, C.c_size_t]),
    ("rvh_asset_write", _st, [_vp, _vp, C.c_size_t]),
    ("rvh_asset_read_positions_async", _st, [_vp, _vp, C.c_size_t, _vp]),
    ("rvh_asset_read_draw", _st, [_vp, _P(T.DrawIndirect)]),
    ("rvh_asset_read_grid", _st, [_vp, _P(C.c_int64), C.c_size_t]),
    ("rvh_step", _st, [_vp, _P(T.Frame), _vp]),
    ("rvh_step_noalloc", _st, [_vp, _P(T.Frame), _vp]),
    ("rvh_batch_create", _st, [_vp, _P(_vp), C.c_int32, _vp, _P(_vp)]),
    ("rvh_batch_destroy", _st, [_vp]),
    ("rvh_batch_step", _st, [_vp, _P(T.Frame), _vp]),
    ("rvh_batch_check", _st, [_vp]),
    ("rvh_batch_finish", _st, [_vp, _vp]),
    ("rvh_batch_info", _st, [_vp, _P(C.c_int32), _P(C.c_int32), _P(C.c_int32), _P(C.c_int64)]),
    ("rvh_batch_read_positions_async", _st, [_vp, _vp, C.c_size_t, _vp]),
    ("rvh_batch_step_read_positions", _st, [_vp, _vp, _vp, C.c_size_t, _vp]),
    ("rvh_batch_positions_wait", _st, [_vp]),
    ("rvh_batch_box_stats", _st, [_vp, _P(C.c_uint32)]),
    ("rvh_batch_h2d_bytes", _st, [_vp, _P(C.c_uint64)]),
    ("rvh_batch_timing_enable", _st, [_vp, C.c_int32]),
    ("rvh_batch_timing_read", _st, [_vp, _P(C.c_double), _P(C.c_int32)]),
    ("rvh_tune_batch", _st, [_vp, _P(_vp), C.c_int32, _vp, _vp, _vp]),
    ("rvh_tune_lookup", _st, [_P(_vp), C.c_int32, C.c_int32, _vp]),
    ("rvh_server_create", _st, [_vp, _vp, _P(_vp)]),
    ("rvh_server_destroy", _st, [_vp]),
    ("rvh_server_add_character", _st, [_vp, _vp, _vp, C.c_float, _P(C.c_int32)]),
    ("rvh_server_character_steps", _st, [_vp, C.c_int32, _P(C.c_int64)]),
    ("rvh_server_run", _st, [_vp, _vp, C.c_int32, _vp, _vp]),
    ("rvh_adjoint", _st, [_vp, _P(T.Frame), C.c_int32, C.c_int32, _P(C.c_float), _P(C.c_double),
                          _P(C.c_float), _P(C.c_float), _P(C.c_float)]),
    ("rvh_generate_head", _st, [_vp, _vp, _P(C.c_float), _P(T.SimParams), _P(T.Collider), _P(C.c_int32)]),
    ("rvh_wind_at", _st, [_vp, C.c_int64, C.c_float, _P(C.c_float)]),
    ("rvh_sphere_on_orbit", _st, [_vp, C.c_float, _P(T.Collider)]),
    ("rvh_tess_desc_reference", _st, [_vp]),
    ("rvh_asset_tessellate", _st, [_vp, _vp, _vp, _vp, _vp]),
    ("rvh_shade_desc_reference", _st, [_vp]),
    ("rvh_shade_fragments", _st, [_vp, C.c_int64, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp, _vp]),
    ("rvh_asset_shade", _st, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("rvh_render_image", _st, [_vp, C.c_int64, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp, _vp]),
    ("rvh_asset_health", _st, [_vp, _vp]),
    ("rvh_asset_snapshot_bytes", _st, [_vp, _P(C.c_uint64)]),
    ("rvh_asset_snapshot", _st, [_vp, _vp, C.c_uint64]),
    ("rvh_asset_restore", _st, [_vp, _vp, C.c_uint64, C.c_int32, _P(_vp)]),
    ("rvh_asset_render_hair", _st, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp, _vp, _vp]),
    ("rvh_mesh_load_obj", _st, [C.c_char_p, _P(_vp)]),
    ("rvh_mesh_from_triangles", _st, [_P(C.c_float), _P(C.c_float), C.c_int32, _P(_vp)]),
    ("rvh_mesh_destroy", None, [_vp]),
    ("rvh_mesh_info", _st, [_vp, _P(C.c_int32), _P(C.c_double)]),
    ("rvh_mesh_triangles", _st, [_vp, _P(C.c_float), _P(C.c_float)]),
    ("rvh_mesh_sample_roots", _st, [_vp, _vp, _P(C.c_float), _P(C.c_float)]),
    ("rvh_libc_rand_sequence", _st, [C.c_uint32, C.c_int32, _P(C.c_int32)]),
    ("rvh_rng_u64", C.c_uint64, [C.c_uint64, C.c_uint64]),
    ("rvh_rng_uniform", C.c_double, [C.c_uint64, C.c_uint64]),
    ("rvh_rng_normal", C.c_double, [C.c_uint64, C.c_uint64]),
]

_lib = None


class RvhError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("rvh status %d: %s" % (status, msg))
        self.status = status


def load(path=LIB_PATH):
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError("librvh.so is not built (%s); run realtime-vulkan-hair_gb300/build.py" % path)
        lib = C.CDLL(path)
        for name, res, args in PROTOTYPES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status):
    if status != 0:
        msg = load().rvh_last_error()
        raise RvhError(status, msg.decode() if msg else "")
    return status
