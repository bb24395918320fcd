"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this.
It exposes the FP64 oracle, its FP32 twin, the FP64 adjoint, and (where the
reference checkout exists) the reference's own shader compiled as C++.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.join(HERE, "..", "realtime-vulkan-hair_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from rvh import types as T  # noqa: E402  (layouts only)

from . import build as _build  # noqa: E402
from . import build_ref as _build_ref  # noqa: E402

_lib = None
_ref = None

_P = C.POINTER


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        l = C.CDLL(path)
        common = [C.c_int, C.c_int, _P(C.c_float), _P(C.c_float), _P(T.SimParams), _P(T.Frame), _P(T.Collider),
                  C.c_int, C.c_int, C.c_int, _P(C.c_int64)]
        l.oracle_run_f64.argtypes = [_P(C.c_double)] + common
        l.oracle_run_f32.argtypes = [_P(C.c_float)] + common
        l.oracle_tess.argtypes = [_P(C.c_float), C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                  C.c_float, C.c_int, _P(C.c_float), _P(C.c_float)]
        l.oracle_tess.restype = C.c_int
        f4 = _P(C.c_float)
        l.oracle_shade_fragments.argtypes = [C.c_longlong, f4, f4, f4, C.c_int, C.c_int, C.c_int, f4]
        l.oracle_shade_camera.argtypes = [f4] * 6
        l.oracle_opacity_fragments.argtypes = [C.c_longlong, f4, f4, C.c_int, C.c_int, f4]
        l.oracle_shade_maps.argtypes = [f4, C.c_longlong, f4, C.c_int, C.c_int, f4, f4]
        l.oracle_shade_vertex_inputs.argtypes = [f4, f4, C.c_int, C.c_int, C.c_int, C.c_int, f4, f4, f4, f4]
        l.oracle_render_image.argtypes = [f4, f4, C.c_longlong, f4, f4, C.c_int, C.c_int, f4]
        l.oracle_shade_maps_quads.argtypes = [f4, C.c_int, C.c_int, C.c_int, f4, f4, C.c_int, C.c_int, C.c_int, f4, f4]
        l.oracle_render_hair.argtypes = [f4, f4, C.c_int, C.c_int, C.c_int, C.c_int, f4, f4, f4, f4, f4, f4, C.c_int,
                                         C.c_int, C.c_int, C.c_int, C.c_int, f4, _P(C.c_uint32)]
        l.oracle_render_hair_blend.argtypes = [f4, f4, C.c_int, C.c_int, C.c_int, C.c_int, f4, f4, f4, f4, f4, f4,
                                               C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, f4, f4, _P(C.c_uint32)]
        l.oracle_render_hair_blend.restype = C.c_int
        for f in (l.oracle_shade_fragments, l.oracle_shade_camera, l.oracle_opacity_fragments, l.oracle_shade_maps, l.oracle_shade_vertex_inputs,
                  l.oracle_render_image, l.oracle_render_hair, l.oracle_shade_maps_quads):
            f.restype = C.c_int
        l.oracle_run_head_f64.argtypes = [_P(C.c_double)] + common + [_P(C.c_float), _P(C.c_float)]
        l.oracle_run_head_f32.argtypes = [_P(C.c_float)] + common + [_P(C.c_float), _P(C.c_float)]
        adj = [_P(C.c_double), C.c_int, C.c_int, _P(C.c_double), _P(C.c_double), _P(T.SimParams), _P(T.Frame),
               _P(T.Collider), C.c_int, C.c_int, _P(C.c_double), C.c_int, _P(C.c_double)]
        l.oracle_adjoint_f64.argtypes = adj + [_P(C.c_double), _P(C.c_double), _P(C.c_double)]
        l.oracle_loss_f64.argtypes = adj
        for f in (l.oracle_run_f64, l.oracle_run_f32, l.oracle_run_head_f64, l.oracle_run_head_f32,
                  l.oracle_adjoint_f64, l.oracle_loss_f64):
            f.restype = C.c_int
        l.oracle_max_threads.restype = C.c_int
        l.oracle_generate_head.argtypes = [_P(T.HeadDesc), C.c_void_p, _P(C.c_float), _P(T.SimParams),
                                           _P(T.Collider), _P(C.c_int32)]
        l.oracle_generate_head.restype = C.c_int
        l.oracle_wind_at.argtypes = [_P(T.WindDesc), C.c_int64, C.c_float, _P(C.c_float)]
        l.oracle_wind_at.restype = C.c_int
        _lib = l
    return _lib


def _fptr(a, ct):
    return None if a is None else a.ctypes.data_as(_P(ct))


def _cols(colliders, n_steps):
    """colliders: list of Collider (same every step) or list (per step) of lists."""
    if colliders and isinstance(colliders[0], (list, tuple)):
        rows = list(colliders)
        assert len(rows) == n_steps
    else:
        rows = [list(colliders)] * n_steps
    ncol = len(rows[0]) if rows else 0
    return T.colliders_array(rows), ncol


def _frames(frames, n_steps):
    if isinstance(frames, T.Frame):
        frames = [frames] * n_steps
    assert len(frames) == n_steps
    return T.frames_array(frames)


def run(state, n_points, rest, params, frames, colliders, n_steps, strand_wind=None, threads=1,
        want_grid=False, heads=None, root_rest=None):
    """Advance `state` (float64 -> FP64 oracle, float32 -> FP32 twin) in place.

    state: (ns, 3*n_points, 4) array in the Strand record layout.
    heads (n_steps, 16) column-major head poses and root_rest (ns, 3): each step
    first places the roots at heads[s] * root_rest (kinematic head).
    Returns the last step's grid (nx*ny*nz, 4) int64 when want_grid."""
    assert state.flags.c_contiguous
    ns = state.shape[0]
    rest = np.ascontiguousarray(rest, np.float32)
    wind = None if strand_wind is None else np.ascontiguousarray(strand_wind, np.float32)
    fr = _frames(frames, n_steps)
    cols, ncol = _cols(colliders, n_steps)
    grid = None
    if want_grid and params.grid_enabled:
        d = params.grid_dims
        grid = np.zeros((d[0] * d[1] * d[2], 4), np.int64)
    head_args = ()
    suffix = ""
    if heads is not None:
        hd = np.ascontiguousarray(heads, np.float32).reshape(n_steps, 16)
        rr = np.ascontiguousarray(root_rest, np.float32).reshape(ns, 3)
        head_args = (_fptr(hd, C.c_float), _fptr(rr, C.c_float))
        suffix = "head_"
    if state.dtype == np.float64:
        fn, ptr = getattr(lib(), "oracle_run_%sf64" % suffix), _fptr(state, C.c_double)
    elif state.dtype == np.float32:
        fn, ptr = getattr(lib(), "oracle_run_%sf32" % suffix), _fptr(state, C.c_float)
    else:
        raise TypeError(state.dtype)
    rc = fn(ptr, ns, n_points, _fptr(rest, C.c_float), _fptr(wind, C.c_float), C.byref(params), fr, cols, ncol,
            n_steps, threads, _fptr(grid, C.c_int64), *head_args)
    if rc != 0:
        raise RuntimeError("oracle_run failed: %d" % rc)
    return grid


def run_group(states, n_points, rests, params, frames, colliders, n_steps):
    """Advance a group of assets sharing one grid in place (hair_oracle.hpp
    step_group): states (all float64 -> FP64 oracle, all float32 -> FP32 twin),
    each (ns_k, 3*n_k, 4); n_points, rests and params per member; frames and
    colliders shared."""
    nm = len(states)
    dt = states[0].dtype
    assert all(st.dtype == dt and st.flags.c_contiguous for st in states)
    ct = C.c_double if dt == np.float64 else C.c_float
    rests = [np.ascontiguousarray(r, np.float32) for r in rests]
    sp = (_P(ct) * nm)(*[st.ctypes.data_as(_P(ct)) for st in states])
    ns = (C.c_int * nm)(*[st.shape[0] for st in states])
    nn = (C.c_int * nm)(*n_points)
    rp = (_P(C.c_float) * nm)(*[r.ctypes.data_as(_P(C.c_float)) for r in rests])
    pa = (T.SimParams * nm)(*params)
    fr = _frames(frames, n_steps)
    cols, ncol = _cols(colliders, n_steps)
    fn = lib().oracle_run_group_f64 if dt == np.float64 else lib().oracle_run_group_f32
    rc = fn(nm, sp, ns, nn, rp, pa, fr, cols, ncol, n_steps)
    if rc != 0:
        raise RuntimeError("oracle_run_group failed: %d" % rc)


def adjoint(state0, n_points, rest, params, frames, colliders, n_steps, targets, strand_wind=None, threads=1):
    """FP64 adjoint: returns (loss, d_wind (ns,3), d_rest (ns,), d_v0 (ns,n,3))."""
    ns = state0.shape[0]
    s0 = np.ascontiguousarray(state0, np.float64)
    rest = np.ascontiguousarray(rest, np.float64)
    wind = np.zeros((ns, 3)) if strand_wind is None else np.ascontiguousarray(strand_wind, np.float64)
    tg = np.ascontiguousarray(targets, np.float64)
    fr = _frames(frames, n_steps)
    cols, ncol = _cols(colliders, n_steps)
    loss = np.zeros(1)
    dw = np.zeros((ns, 3))
    dr = np.zeros(ns)
    dv = np.zeros((ns, n_points, 3))
    rc = lib().oracle_adjoint_f64(_fptr(s0, C.c_double), ns, n_points, _fptr(rest, C.c_double),
                                  _fptr(wind, C.c_double), C.byref(params), fr, cols, ncol, n_steps,
                                  _fptr(tg, C.c_double), threads, _fptr(loss, C.c_double), _fptr(dw, C.c_double),
                                  _fptr(dr, C.c_double), _fptr(dv, C.c_double))
    if rc != 0:
        raise RuntimeError("oracle_adjoint failed: %d" % rc)
    return loss[0], dw, dr, dv


def loss(state0, n_points, rest, params, frames, colliders, n_steps, targets, strand_wind=None, threads=1):
    ns = state0.shape[0]
    s0 = np.ascontiguousarray(state0, np.float64)
    rest = np.ascontiguousarray(rest, np.float64)
    wind = np.zeros((ns, 3)) if strand_wind is None else np.ascontiguousarray(strand_wind, np.float64)
    tg = np.ascontiguousarray(targets, np.float64)
    fr = _frames(frames, n_steps)
    cols, ncol = _cols(colliders, n_steps)
    out = np.zeros(1)
    rc = lib().oracle_loss_f64(_fptr(s0, C.c_double), ns, n_points, _fptr(rest, C.c_double),
                               _fptr(wind, C.c_double), C.byref(params), fr, cols, ncol, n_steps,
                               _fptr(tg, C.c_double), threads, _fptr(out, C.c_double))
    if rc != 0:
        raise RuntimeError("oracle_loss failed: %d" % rc)
    return out[0]


class SceneGen:
    """The seeded synthetic inputs (include/rvh_scene.h) from the oracle's own
    statement of them (scene_oracle.hpp): rvh.configs builds a workload with
    it when given gen=SceneGen(), so the CPU timing arm of bench.py never
    maps the CUDA library.  Same calls and results as rvh.api's."""

    @staticmethod
    def generate_head(**kw):
        d = T.head_desc(**kw)
        ns, n = d.n_strands, d.n_points
        rec = np.empty((ns, 3 * n, 4), np.float32)
        rest = np.empty(max(ns, 1), np.float32)
        p = T.SimParams()
        cols = (T.Collider * T.MAX_COLLIDERS)()
        nc = C.c_int32()
        rc = lib().oracle_generate_head(C.byref(d), rec.ctypes.data_as(C.c_void_p), _fptr(rest, C.c_float),
                                        C.byref(p), cols, C.byref(nc))
        if rc != 0:
            raise RuntimeError("oracle_generate_head failed: %d" % rc)
        return rec, rest[:ns], p, [cols[i] for i in range(nc.value)]

    @staticmethod
    def wind_at(desc, step, t):
        out = (C.c_float * 3)()
        if lib().oracle_wind_at(C.byref(desc), step, t, out) != 0:
            raise RuntimeError("oracle_wind_at failed")
        return tuple(out)


def max_threads():
    return lib().oracle_max_threads()


# ---- the reference's own shader compiled as C++ (only where the checkout exists) ----

def ref_available():
    return _build_ref.available()


def ref_lib():
    global _ref
    if _ref is None:
        path = _build_ref.build()
        if path is None:
            return None
        l = C.CDLL(path)
        l.ref_run.argtypes = [_P(C.c_float), C.c_int, _P(C.c_float), _P(C.c_float), C.c_int, _P(C.c_int32),
                              _P(C.c_uint32)]
        l.ref_run.restype = C.c_int
        l.ref_collider.argtypes = [_P(C.c_float)] * 4
        l.ref_translate.argtypes = [_P(C.c_float)] * 2
        _ref = l
    return _ref


def ref_collider(trans, rot_deg, scale):
    out = np.zeros(48, np.float32)
    a = [np.ascontiguousarray(x, np.float32) for x in (trans, rot_deg, scale)]
    ref_lib().ref_collider(*[_fptr(x, C.c_float) for x in a], _fptr(out, C.c_float))
    return out


def ref_translate(flat48, delta):
    out = np.ascontiguousarray(flat48, np.float32).copy()
    d = np.ascontiguousarray(delta, np.float32)
    ref_lib().ref_translate(_fptr(out, C.c_float), _fptr(d, C.c_float))
    return out


def ref_run(strands, colliders_steps, times, want_grid=False):
    """strands: (ns, 30, 4) float32, advanced in place; colliders_steps: (steps, 6, 48);
    times: (steps, 2).  Returns (grid int32 (64^3,4) or None, draw uint32[4])."""
    assert strands.dtype == np.float32 and strands.flags.c_contiguous
    cs = np.ascontiguousarray(colliders_steps, np.float32)
    tm = np.ascontiguousarray(times, np.float32)
    steps = tm.shape[0]
    grid = np.zeros((64 ** 3, 4), np.int32) if want_grid else None
    draw = np.zeros(4, np.uint32)
    rc = ref_lib().ref_run(_fptr(strands, C.c_float), strands.shape[0], _fptr(cs, C.c_float), _fptr(tm, C.c_float),
                           steps, _fptr(grid, C.c_int32), _fptr(draw, C.c_uint32))
    if rc != 0:
        raise RuntimeError("ref_run failed")
    return grid, draw


def tessellate(records, n_points, n_lines=12, n_segments=42, clump_radius=0.5, root_width=0.02, tip_width=0.01,
               sin_mode=1, frames=False):
    """Oracle tessellation: (ns, n_lines, n_segments+1, 4) float32 and, with
    frames, (ns, n_points-1, 3, 4)."""
    rec = np.ascontiguousarray(records, np.float32)
    ns = rec.shape[0]
    out = np.zeros((ns, n_lines, n_segments + 1, 4), np.float32)
    fr = np.zeros((ns, n_points - 1, 3, 4), np.float32) if frames else None
    rc = lib().oracle_tess(_fptr(rec, C.c_float), ns, n_points, n_lines, n_segments, clump_radius, root_width,
                           tip_width, sin_mode, _fptr(out, C.c_float), _fptr(fr, C.c_float))
    if rc != 0:
        raise RuntimeError("oracle_tess failed: %d" % rc)
    return (out, fr) if frames else out


# ---- hair shading (shade_oracle.hpp) ---------------------------------------------------------

def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _check(rc, name):
    if rc != 0:
        raise RuntimeError("%s failed: %d" % (name, rc))


def shade_fragments(inputs, depth, opacity, sin_mode=1):
    """hair.frag per fragment: inputs (n, 24), depth (h, w), opacity (h, w, 4) -> (n, 4)."""
    inp, dep, opa = _f32(inputs), _f32(depth), _f32(opacity)
    n = inp.shape[0]
    h, w = dep.shape
    out = np.zeros((n, 4), np.float32)
    _check(lib().oracle_shade_fragments(n, _fptr(inp, C.c_float), _fptr(dep, C.c_float), _fptr(opa, C.c_float), w, h,
                                        sin_mode, _fptr(out, C.c_float)), "oracle_shade_fragments")
    return out


def opacity_fragments(inputs, depth):
    """hairOpacity.frag per fragment: (n, 4) = layers 1-3 (0 or 0.3) and z0."""
    inp, dep = _f32(inputs), _f32(depth)
    h, w = dep.shape
    out = np.zeros((inp.shape[0], 4), np.float32)
    _check(lib().oracle_opacity_fragments(inp.shape[0], _fptr(inp, C.c_float), _fptr(dep, C.c_float), w, h,
                                          _fptr(out, C.c_float)), "oracle_opacity_fragments")
    return out


def _mats(desc):
    return [_f32(np.array(list(getattr(desc, f)), np.float32)) for f in
            ("camera_view", "camera_proj", "light_view", "light_proj")]


def shade_camera(desc):
    """(lvp (16,), cam_pos (3,), light_pos (3,)) of a ShadeDesc."""
    cv, _, lv, lp = _mats(desc)
    lvp = np.zeros(16, np.float32)
    cam = np.zeros(3, np.float32)
    light = np.zeros(3, np.float32)
    _check(lib().oracle_shade_camera(*[_fptr(a, C.c_float) for a in (cv, lv, lp, lvp, cam, light)]),
           "oracle_shade_camera")
    return lvp, cam, light


def shade_maps(vertices, desc, n_lines=None, n_segments=None, sin_mode=1):
    """Light depth (h, w) and deep opacity (h, w, 4) maps of tessellated vertices,
    as desc.map_mode says: hair.geom's quads rasterised in the light's view
    (vertices shaped (ns, n_lines, n_segments + 1, 4)), or one texel per vertex."""
    if getattr(desc, "map_mode", 0) == 1:
        v = _f32(vertices)
        ns, L, S1 = v.shape[0], v.shape[1], v.shape[2]
        _, _, lv, lp = _mats(desc)
        w, h = desc.map_width, desc.map_height
        depth = np.zeros((h, w), np.float32)
        opacity = np.zeros((h, w, 4), np.float32)
        _check(lib().oracle_shade_maps_quads(_fptr(v, C.c_float), ns, L, S1 - 1, _fptr(lv, C.c_float),
                                             _fptr(lp, C.c_float), w, h, sin_mode, _fptr(depth, C.c_float),
                                             _fptr(opacity, C.c_float)), "oracle_shade_maps_quads")
        return depth, opacity
    v = _f32(vertices).reshape(-1, 4)
    lvp, _, _ = shade_camera(desc)
    w, h = desc.map_width, desc.map_height
    depth = np.zeros((h, w), np.float32)
    opacity = np.zeros((h, w, 4), np.float32)
    _check(lib().oracle_shade_maps(_fptr(v, C.c_float), v.shape[0], _fptr(lvp, C.c_float), w, h,
                                   _fptr(depth, C.c_float), _fptr(opacity, C.c_float)), "oracle_shade_maps")
    return depth, opacity


def shade_vertex_inputs(vertices, frames, n_points, n_lines, n_segments, desc):
    """Fragment inputs (n_vertices, 24) of tessellated vertices (ns, L, S+1, 4) and frames (ns, n-1, 3, 4)."""
    v, fr = _f32(vertices), _f32(frames)
    ns = v.shape[0]
    cv, _, lv, lp = _mats(desc)
    out = np.zeros((ns * n_lines * (n_segments + 1), 24), np.float32)
    _check(lib().oracle_shade_vertex_inputs(_fptr(v, C.c_float), _fptr(fr, C.c_float), ns, n_points, n_lines,
                                            n_segments, _fptr(cv, C.c_float), _fptr(lv, C.c_float),
                                            _fptr(lp, C.c_float), _fptr(out, C.c_float)), "oracle_shade_vertex_inputs")
    return out


def render_image(vertices, colors, desc, width, height):
    """Nearest-vertex camera image (height, width, 4)."""
    v, col = _f32(vertices).reshape(-1, 4), _f32(colors).reshape(-1, 4)
    cv, cp, _, _ = _mats(desc)
    img = np.zeros((height, width, 4), np.float32)
    _check(lib().oracle_render_image(_fptr(v, C.c_float), _fptr(col, C.c_float), v.shape[0], _fptr(cv, C.c_float),
                                     _fptr(cp, C.c_float), width, height, _fptr(img, C.c_float)),
           "oracle_render_image")
    return img


# the reference framebuffer's clear colour (src/Renderer.cpp:2235)
CLEAR_RGBA = np.array([101.0 / 255.0, 129.0 / 255.0, 140.0 / 255.0, 1.0], np.float32)


def render_hair(vertices, frames, n_points, n_lines, n_segments, desc, depth, opacity, width, height, sin_mode=1):
    """hair.geom's quads rasterised into a (height, width, 4) image shaded by
    hair.frag, and per pixel the nearest fragment's segment id (0xffffffff:
    none).  desc.image_mode 1 (blend): the pipeline's in-order blending from the
    reference's clear colour; 0: the nearest fragment's colour."""
    v, fr = _f32(vertices), _f32(frames)
    dep, opa = _f32(depth), _f32(opacity)
    ns = v.shape[0]
    cv, cp, lv, lp = _mats(desc)
    img = np.zeros((height, width, 4), np.float32)
    ids = np.zeros((height, width), np.uint32)
    mh, mw = dep.shape
    args = [_fptr(v, C.c_float), _fptr(fr, C.c_float), ns, n_points, n_lines, n_segments,
            *[_fptr(a, C.c_float) for a in (cv, cp, lv, lp, dep, opa)], mw, mh, width, height, sin_mode]
    if getattr(desc, "image_mode", 0) == 1:
        _check(lib().oracle_render_hair_blend(*args, _fptr(CLEAR_RGBA, C.c_float), _fptr(img, C.c_float),
                                              ids.ctypes.data_as(_P(C.c_uint32))), "oracle_render_hair_blend")
    else:
        _check(lib().oracle_render_hair(*args, _fptr(img, C.c_float), ids.ctypes.data_as(_P(C.c_uint32))),
               "oracle_render_hair")
    return img, ids
