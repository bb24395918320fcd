"""Python host-side mirror of the C ABI: Context, Asset (the reference's Hair),
Batch, and the scene helpers.  Every call goes through librvh.so."""
import ctypes as C
import os

import numpy as np

from . import types as T
from ._lib import check, load

_P = C.POINTER


class ContextDesc(C.Structure):
    _fields_ = [("device", C.c_int32), ("math", C.c_int32), ("hbm_budget_bytes", C.c_uint64)]


class AssetDesc(C.Structure):
    _fields_ = [("n_strands", C.c_int32), ("n_points", C.c_int32), ("strands", C.c_void_p),
                ("strands_location", C.c_int32), ("uniform_rest_length", C.c_float),
                ("rest_lengths", _P(C.c_float)), ("strand_wind", _P(C.c_float)),
                ("lanes_per_strand", C.c_int32), ("reserved", C.c_int32)]


class Health(C.Structure):
    _fields_ = [("nonfinite", C.c_uint64), ("max_speed", C.c_float), ("max_length_error", C.c_float),
                ("worst_strand", C.c_int32), ("reserved", C.c_int32)]


class SnapshotHeader(C.Structure):
    _fields_ = [("magic", C.c_char * 8), ("version", C.c_uint32), ("header_bytes", C.c_uint32),
                ("total_bytes", C.c_uint64), ("n_strands", C.c_int32), ("n_points", C.c_int32), ("flags", C.c_uint32),
                ("n_colliders", C.c_int32), ("lanes_per_strand", C.c_int32), ("reserved", C.c_int32),
                ("params", T.SimParams), ("colliders", T.Collider * 8), ("head", C.c_float * 16)]


class BatchDesc(C.Structure):
    _fields_ = [("lanes_per_strand", C.c_int32), ("strands_per_tile", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("use_graph", C.c_int32), ("full_steps", C.c_int32), ("reserved", C.c_int32)]


HeadDesc = T.HeadDesc   # layouts in rvh/types.py (shared with the oracle)
WindDesc = T.WindDesc


class TuneDesc(C.Structure):
    _fields_ = [("steps", C.c_int32), ("tune_grid", C.c_int32), ("use_cache", C.c_int32), ("n_grid_res", C.c_int32),
                ("grid_res", C.c_int32 * 8)]


class TuneResult(C.Structure):
    _fields_ = [("lanes_per_strand", C.c_int32), ("strands_per_tile", C.c_int32), ("grid_res", C.c_int32),
                ("n_tried", C.c_int32), ("best_ms", C.c_float), ("tried_lanes", C.c_int32 * 96),
                ("tried_tile", C.c_int32 * 96), ("tried_res", C.c_int32 * 96), ("tried_ms", C.c_float * 96)]

    def table(self):
        return [(self.tried_lanes[i], self.tried_tile[i], self.tried_res[i], self.tried_ms[i])
                for i in range(self.n_tried)]


def tune(ctx, assets, frames, steps=3, grid_res=(), use_cache=False):
    d = TuneDesc()
    d.steps = steps
    d.tune_grid = 1 if grid_res else 0
    d.use_cache = 1 if use_cache else 0
    d.n_grid_res = len(grid_res)
    for i, r in enumerate(grid_res):
        d.grid_res[i] = r
    arr = (C.c_void_p * len(assets))(*[a.h.value for a in assets])
    fr = (T.Frame * len(frames))(*frames)
    out = TuneResult()
    check(ctx.lib.rvh_tune_batch(ctx.h, arr, len(assets), fr, C.byref(d), C.byref(out)))
    return out


class Orbit(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("orbit_radius", C.c_float), ("omega", C.c_float),
                ("phase", C.c_float), ("sphere_radius", C.c_float)]


class ServerDesc(C.Structure):
    _fields_ = [("max_active", C.c_int32), ("lanes_per_strand", C.c_int32), ("pipeline_depth", C.c_int32),
                ("steps_per_launch", C.c_int32), ("scratch_budget_bytes", C.c_uint64)]


class Request(C.Structure):
    _fields_ = [("character", C.c_int32), ("n_steps", C.c_int32), ("arrival_s", C.c_double)]


class RequestResult(C.Structure):
    _fields_ = [("admit_s", C.c_double), ("done_s", C.c_double), ("max_step_ms", C.c_float),
                ("steps_done", C.c_int32), ("status", C.c_int32), ("reserved", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("requests", C.c_int64), ("steps", C.c_int64), ("point_steps", C.c_int64), ("launches", C.c_int32),
                ("max_active", C.c_int32), ("wall_s", C.c_double), ("point_steps_per_s", C.c_double),
                ("step_ms_p50", C.c_double), ("step_ms_p99", C.c_double), ("step_ms_p999", C.c_double),
                ("request_ms_p50", C.c_double), ("request_ms_p99", C.c_double), ("queue_ms_p50", C.c_double),
                ("queue_ms_p99", C.c_double), ("mean_batch", C.c_double), ("admission_waits", C.c_int64),
                ("scratch_used_bytes", C.c_uint64), ("gpu_busy_frac", C.c_double), ("host_ms_per_launch", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


MATH_FAST = 0
MATH_EXACT = 1


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _fp(a):
    return None if a is None else a.ctypes.data_as(_P(C.c_float))


class PinnedBuffer:
    """Page-locked host memory from the library (for asynchronous copies)."""

    def __init__(self, nbytes):
        self.lib = load()
        p = C.c_void_p()
        check(self.lib.rvh_pinned_alloc(nbytes, C.byref(p)))
        self.ptr, self.nbytes = p.value, nbytes

    def array(self, shape, dtype=np.float32):
        buf = (C.c_char * self.nbytes).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    def close(self):
        if self.ptr:
            self.lib.rvh_pinned_free(C.c_void_p(self.ptr))
            self.ptr = None


class Context:
    def __init__(self, device=0, math=MATH_FAST, hbm_budget_bytes=0):
        self.lib = load()
        d = ContextDesc(device, math, hbm_budget_bytes)
        h = C.c_void_p()
        check(self.lib.rvh_context_create(C.byref(d), C.byref(h)))
        self.h = h
        self.math = math

    def close(self):
        if self.h:
            self.lib.rvh_context_destroy(self.h)
            self.h = None

    def synchronize(self):
        check(self.lib.rvh_context_synchronize(self.h))

    def memory(self):
        u, b = C.c_uint64(), C.c_uint64()
        check(self.lib.rvh_context_memory(self.h, C.byref(u), C.byref(b)))
        return u.value, b.value

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Asset:
    """One hair asset: the reference's Hair buffers (Strand.h:61-80) on the GPU."""

    def __init__(self, ctx, records, n_points, rest=None, uniform_rest=0.0, strand_wind=None, lanes=0,
                 location=T.MEM_HOST, device_ptr=None):
        self.ctx = ctx
        self.lib = ctx.lib
        if device_ptr is not None:
            n_strands = int(records)
            src = C.c_void_p(device_ptr)
        else:
            rec = _f32(records).reshape(-1)
            n_strands = rec.size // (12 * n_points)
            assert n_strands * 12 * n_points == rec.size
            src = rec.ctypes.data_as(C.c_void_p)
            self._keep = rec
        self.n_strands, self.n_points = n_strands, n_points
        rest_a = None if rest is None else _f32(rest)
        wind_a = None if strand_wind is None else _f32(strand_wind).reshape(-1)
        d = AssetDesc(n_strands, n_points, src, location, uniform_rest, _fp(rest_a), _fp(wind_a), lanes, 0)
        h = C.c_void_p()
        check(self.lib.rvh_asset_create(ctx.h, C.byref(d), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.rvh_asset_destroy(self.h)
            self.h = None

    def health(self):
        """Non-finite count, largest speed and inextensibility error (rvh_asset_health)."""
        h = Health()
        check(self.lib.rvh_asset_health(self.h, C.byref(h)))
        return h

    def snapshot(self):
        """The asset's whole simulation state as bytes (rvh_asset_snapshot)."""
        n = C.c_uint64()
        check(self.lib.rvh_asset_snapshot_bytes(self.h, C.byref(n)))
        buf = (C.c_ubyte * n.value)()
        check(self.lib.rvh_asset_snapshot(self.h, buf, n.value))
        return bytes(buf)

    @classmethod
    def restore(cls, ctx, data, lanes=0):
        """A new asset in ctx from snapshot bytes (rvh_asset_restore)."""
        buf = (C.c_ubyte * len(data)).from_buffer_copy(data)
        h = C.c_void_p()
        check(ctx.lib.rvh_asset_restore(ctx.h, buf, len(data), lanes, C.byref(h)))
        self = cls.__new__(cls)
        self.ctx, self.lib, self.h = ctx, ctx.lib, h
        ns, npts = C.c_int32(), C.c_int32()
        check(ctx.lib.rvh_asset_strand_count(h, C.byref(ns), C.byref(npts)))
        self.n_strands, self.n_points = ns.value, npts.value
        return self

    def set_params(self, p):
        check(self.lib.rvh_asset_set_params(self.h, C.byref(p)))

    def set_colliders(self, cols):
        arr = (T.Collider * max(1, len(cols)))(*cols)
        check(self.lib.rvh_asset_set_colliders(self.h, arr, len(cols)))

    def share_grid(self, owner):
        """Splat into and gather from `owner`'s grid (None: a grid of its own again)."""
        check(self.lib.rvh_asset_share_grid(self.h, owner.h if owner is not None else None))

    def set_head_transform(self, m):
        """m: 4x4 head pose (numpy, row-major as written; passed column-major), or None to stop."""
        if m is None:
            check(self.lib.rvh_asset_set_head_transform(self.h, None))
            return
        cm = np.ascontiguousarray(np.asarray(m, np.float32).T)
        check(self.lib.rvh_asset_set_head_transform(self.h, _fp(cm)))

    def step(self, frame, stream=None):
        check(self.lib.rvh_step(self.h, C.byref(frame), stream))

    def tessellate(self, vertices_ptr, frames_ptr=None, desc=None, stream=None):
        """Writes n_strands * n_lines * (n_segments+1) float4 vertices (and, with
        frames_ptr, (n_points-1) * 3 float4 frames per strand) to device memory."""
        d = desc if desc is not None else tess_desc_reference()
        check(self.lib.rvh_asset_tessellate(self.h, C.byref(d), C.c_void_p(vertices_ptr),
                                            C.c_void_p(frames_ptr) if frames_ptr else None, stream))

    def shade(self, vertices_ptr, frames_ptr, depth_ptr, opacity_ptr, colors_ptr, tess_desc=None, shade_desc=None,
              stream=None):
        """The shadow, opacity and hair passes over this asset's tessellation
        (vertices and frames from tessellate() with the same tess_desc): writes
        the light depth map (map_height x map_width floats), the opacity map
        (the same count of float4) and one float4 colour per vertex."""
        td = tess_desc if tess_desc is not None else tess_desc_reference()
        sd = shade_desc if shade_desc is not None else shade_desc_reference()
        check(self.lib.rvh_asset_shade(self.h, C.byref(td), C.byref(sd), C.c_void_p(vertices_ptr),
                                       C.c_void_p(frames_ptr), C.c_void_p(depth_ptr), C.c_void_p(opacity_ptr),
                                       C.c_void_p(colors_ptr) if colors_ptr else None, stream))

    def render_hair(self, vertices_ptr, frames_ptr, depth_ptr, opacity_ptr, width, height, image_ptr, ids_ptr=None,
                    tess_desc=None, shade_desc=None, stream=None):
        """hair.geom's quads of this asset's tessellation rasterised into a
        height x width float4 image shaded by hair.frag (maps from shade());
        ids_ptr (optional) receives the winning segment per pixel."""
        td = tess_desc if tess_desc is not None else tess_desc_reference()
        sd = shade_desc if shade_desc is not None else shade_desc_reference()
        check(self.lib.rvh_asset_render_hair(self.h, C.byref(td), C.byref(sd), C.c_void_p(vertices_ptr),
                                             C.c_void_p(frames_ptr), C.c_void_p(depth_ptr), C.c_void_p(opacity_ptr),
                                             width, height, C.c_void_p(image_ptr),
                                             C.c_void_p(ids_ptr) if ids_ptr else None, stream))

    def read(self):
        out = np.empty((self.n_strands, 3 * self.n_points, 4), np.float32)
        check(self.lib.rvh_asset_read(self.h, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def write(self, records):
        rec = _f32(records)
        check(self.lib.rvh_asset_write(self.h, rec.ctypes.data_as(C.c_void_p), rec.nbytes))

    def read_grid(self, cells):
        out = np.empty((cells, 4), np.int64)
        check(self.lib.rvh_asset_read_grid(self.h, out.ctypes.data_as(_P(C.c_int64)), out.nbytes))
        return out

    def set_rest_lengths(self, rest):
        r = _f32(rest)
        check(self.lib.rvh_asset_set_rest_lengths(self.h, _fp(r)))

    def set_strand_wind(self, wind):
        w = None if wind is None else _f32(wind).reshape(-1)
        check(self.lib.rvh_asset_set_strand_wind(self.h, _fp(w)))

    def adjoint(self, frames, targets, checkpoint_every=10):
        """Returns (loss, d_wind (ns,3), d_rest (ns,), d_v0 (ns,n,3)) of the tip loss."""
        fr = (T.Frame * len(frames))(*frames)
        tg = _f32(targets).reshape(-1)
        loss = C.c_double()
        dw = np.zeros((self.n_strands, 3), np.float32)
        dr = np.zeros(self.n_strands, np.float32)
        dv = np.zeros((self.n_strands, self.n_points, 3), np.float32)
        check(self.lib.rvh_adjoint(self.h, fr, len(frames), checkpoint_every, _fp(tg), C.byref(loss), _fp(dw),
                                   _fp(dr), _fp(dv)))
        return loss.value, dw, dr, dv

    def read_draw(self):
        d = T.DrawIndirect()
        check(self.lib.rvh_asset_read_draw(self.h, C.byref(d)))
        return (d.vertex_count, d.instance_count, d.first_vertex, d.first_instance)

    def read_positions(self, stream=None):
        out = np.empty((self.n_strands, self.n_points, 4), np.float32)
        check(self.lib.rvh_asset_read_positions_async(self.h, out.ctypes.data_as(C.c_void_p), out.nbytes, stream))
        self.ctx.synchronize()
        return out

    def device_ptr(self):
        p = C.c_void_p()
        check(self.lib.rvh_asset_device_ptr(self.h, C.byref(p)))
        return p.value

    def draw_indirect_ptr(self):
        p = C.c_void_p()
        check(self.lib.rvh_asset_draw_indirect(self.h, C.byref(p)))
        return p.value


class Batch:
    def __init__(self, ctx, assets, lanes=0, strands_per_tile=0, ctas_per_sm=0, use_graph=True, full_steps=False):
        self.ctx = ctx
        self.lib = ctx.lib
        self.assets = list(assets)
        arr = (C.c_void_p * max(1, len(self.assets)))(*[a.h.value for a in self.assets])
        d = BatchDesc(lanes, strands_per_tile, ctas_per_sm, 1 if use_graph else 0, 1 if full_steps else 0, 0)
        h = C.c_void_p()
        check(self.lib.rvh_batch_create(ctx.h, arr, len(self.assets), C.byref(d), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.rvh_batch_destroy(self.h)
            self.h = None

    def step(self, frames, stream=None):
        arr = (T.Frame * max(1, len(frames)))(*frames)
        check(self.lib.rvh_batch_step(self.h, arr, stream))

    def check(self):
        check(self.lib.rvh_batch_check(self.h))

    def finish(self, stream=None):
        check(self.lib.rvh_batch_finish(self.h, stream))

    def read_positions_async(self, host_ptr, nbytes, stream=None):
        check(self.lib.rvh_batch_read_positions_async(self.h, C.c_void_p(host_ptr), nbytes, stream))

    def step_read_positions(self, frames, host_ptr, nbytes, stream=None):
        """One step, then its positions (xyz per point) copied to host_ptr by the
        step's own staging writes; positions_wait() blocks until the copy is done."""
        arr = (T.Frame * max(1, len(frames)))(*frames)
        check(self.lib.rvh_batch_step_read_positions(self.h, arr, C.c_void_p(host_ptr), nbytes, stream))

    def positions_wait(self):
        check(self.lib.rvh_batch_positions_wait(self.h))

    def box_stats(self):
        out = (C.c_uint32 * 4)()
        check(self.lib.rvh_batch_box_stats(self.h, out))
        return {"a_box": out[0], "a_direct": out[1], "b_box": out[2], "b_direct": out[3]}

    def h2d_bytes_per_step(self):
        b = C.c_uint64()
        check(self.lib.rvh_batch_h2d_bytes(self.h, C.byref(b)))
        return b.value

    def timing(self, on=True):
        check(self.lib.rvh_batch_timing_enable(self.h, 1 if on else 0))

    def read_timing(self):
        ms, n = C.c_double(), C.c_int32()
        check(self.lib.rvh_batch_timing_read(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def info(self):
        l, it, ct, pts = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int64()
        check(self.lib.rvh_batch_info(self.h, C.byref(l), C.byref(it), C.byref(ct), C.byref(pts)))
        return {"lanes": l.value, "items": it.value, "ctas": ct.value, "points": pts.value}


class Server:
    """Continuous-batching request loop over resident characters (C++)."""

    def __init__(self, ctx, max_active=16, lanes=8, pipeline_depth=2, scratch_budget_bytes=1 << 30,
                 steps_per_launch=1):
        self.ctx = ctx
        self.lib = ctx.lib
        d = ServerDesc(max_active, lanes, pipeline_depth, steps_per_launch, scratch_budget_bytes)
        h = C.c_void_p()
        check(self.lib.rvh_server_create(ctx.h, C.byref(d), C.byref(h)))
        self.h = h

    def add_character(self, asset, wind=None, dt=1.0 / 60.0):
        i = C.c_int32()
        check(self.lib.rvh_server_add_character(self.h, asset.h, None if wind is None else C.byref(wind), dt,
                                                C.byref(i)))
        return i.value

    def character_steps(self, cid):
        v = C.c_int64()
        check(self.lib.rvh_server_character_steps(self.h, cid, C.byref(v)))
        return v.value

    def run(self, requests):
        """requests: list of (character, n_steps, arrival_s). Returns (results, stats)."""
        n = len(requests)
        arr = (Request * max(1, n))(*[Request(c, k, t) for c, k, t in requests])
        res = (RequestResult * max(1, n))()
        st = ServerStats()
        status = self.lib.rvh_server_run(self.h, arr, n, res, C.byref(st))
        return status, [res[i] for i in range(n)], st

    def close(self):
        if self.h:
            self.lib.rvh_server_destroy(self.h)
            self.h = None


# ---- scene helpers -------------------------------------------------------------

def reference_params():
    p = T.SimParams()
    check(load().rvh_sim_params_reference(C.byref(p)))
    return p


def collider_from_trs(trans, rot_deg, scale, kind=T.COLLIDER_ELLIPSOID, radius=1.0):
    c = T.Collider()
    t, r, s = _f32(trans), _f32(rot_deg), _f32(scale)
    check(load().rvh_collider_from_trs(_fp(t), _fp(r), _fp(s), kind, radius, C.byref(c)))
    return c


def collider_translate(c, delta):
    out = T.Collider()
    C.memmove(C.byref(out), C.byref(c), C.sizeof(T.Collider))
    d = _f32(delta)
    check(load().rvh_collider_translate(C.byref(out), _fp(d)))
    return out


def collider_follow(c, m):
    """The collider carried by head pose m (4x4, row-major as written)."""
    out = T.Collider()
    cm = np.ascontiguousarray(np.asarray(m, np.float32).T)
    check(load().rvh_collider_follow(C.byref(c), _fp(cm), C.byref(out)))
    return out


def init_strands_reference(roots, normals, n_points, seg, dir_offset=(0.05, 5.0, -2.0)):
    roots, normals, off = _f32(roots), _f32(normals), _f32(dir_offset)
    ns = roots.shape[0]
    out = np.empty((ns, 3 * n_points, 4), np.float32)
    check(load().rvh_init_strands_reference(_fp(roots), _fp(normals), ns, n_points, seg, _fp(off),
                                            out.ctypes.data_as(C.c_void_p)))
    return out


def generate_head(**kw):
    """Returns (records (ns, 3n, 4) f32, rest (ns,), SimParams, [Collider])."""
    d = T.head_desc(**kw)
    ns, n = d.n_strands, d.n_points
    rec = np.empty((ns, 3 * n, 4), np.float32)
    rest = np.empty(max(ns, 1), np.float32)
    p = T.SimParams()
    cols = (T.Collider * T.MAX_COLLIDERS)()
    nc = C.c_int32()
    check(load().rvh_generate_head(C.byref(d), rec.ctypes.data_as(C.c_void_p), _fp(rest), C.byref(p), cols,
                                   C.byref(nc)))
    return rec, rest[:ns], p, [cols[i] for i in range(nc.value)]


def wind_at(desc, step, t):
    out = (C.c_float * 3)()
    check(load().rvh_wind_at(C.byref(desc), step, t, out))
    return tuple(out)


def sphere_on_orbit(orbit, t):
    c = T.Collider()
    check(load().rvh_sphere_on_orbit(C.byref(orbit), t, C.byref(c)))
    return c


# ---- strand tessellation ------------------------------------------------------------
class TessDesc(C.Structure):
    _fields_ = [("n_lines", C.c_int32), ("n_segments", C.c_int32), ("clump_radius", C.c_float),
                ("root_width", C.c_float), ("tip_width", C.c_float), ("reserved", C.c_int32)]


def tess_desc_reference(**kw):
    d = TessDesc()
    check(load().rvh_tess_desc_reference(C.byref(d)))
    for k, v in kw.items():
        setattr(d, k, v)
    return d


# ---- hair shading -----------------------------------------------------------------
class ShadeDesc(C.Structure):
    _fields_ = [("camera_view", C.c_float * 16), ("camera_proj", C.c_float * 16), ("light_view", C.c_float * 16),
                ("light_proj", C.c_float * 16), ("map_width", C.c_int32), ("map_height", C.c_int32),
                ("map_mode", C.c_int32), ("image_mode", C.c_int32)]


SHADE_MAPS_VERTICES = 0
SHADE_MAPS_QUADS = 1
IMAGE_NEAREST = 0
IMAGE_BLEND = 1


def shade_desc_reference(**kw):
    d = ShadeDesc()
    check(load().rvh_shade_desc_reference(C.byref(d)))
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def shade_fragments(ctx, n, inputs_ptr, depth_ptr, opacity_ptr, map_width, map_height, colors_ptr, stream=None):
    """hair.frag for n fragments: inputs n x 24 floats, maps as rvh_asset_shade
    writes them, colors n float4 (all device pointers)."""
    check(load().rvh_shade_fragments(ctx.h, n, C.c_void_p(inputs_ptr), C.c_void_p(depth_ptr),
                                     C.c_void_p(opacity_ptr), map_width, map_height, C.c_void_p(colors_ptr), stream))


def render_image(ctx, n_vertices, vertices_ptr, colors_ptr, width, height, image_ptr, shade_desc=None, stream=None):
    """Nearest-vertex camera image (height x width float4) of shaded vertices."""
    sd = shade_desc if shade_desc is not None else shade_desc_reference()
    check(load().rvh_render_image(ctx.h, n_vertices, C.c_void_p(vertices_ptr), C.c_void_p(colors_ptr), C.byref(sd),
                                  width, height, C.c_void_p(image_ptr), stream))


# ---- scalp meshes and root sampling ----------------------------------------------
MESH_ROOTS_REFERENCE = 0
MESH_ROOTS_AREA = 1
ROOT_NORMAL_FIRST_CORNER = 0
ROOT_NORMAL_INTERPOLATED = 1


class MeshRootsDesc(C.Structure):
    _fields_ = [("mode", C.c_int32), ("n_roots", C.c_int32), ("seed", C.c_uint64), ("normal_mode", C.c_int32),
                ("reserved", C.c_int32)]


class Mesh:
    """A triangle mesh in the reference's face-vertex form (rvh_mesh)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    @classmethod
    def load_obj(cls, path):
        h = C.c_void_p()
        check(load().rvh_mesh_load_obj(os.fsencode(path), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_triangles(cls, positions, normals):
        p, n = _f32(positions).reshape(-1, 9), _f32(normals).reshape(-1, 9)
        h = C.c_void_p()
        check(load().rvh_mesh_from_triangles(_fp(p), _fp(n), p.shape[0], C.byref(h)))
        return cls(h.value)

    def close(self):
        if self._h and self._h.value:
            load().rvh_mesh_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        nt, area = C.c_int32(), C.c_double()
        check(load().rvh_mesh_info(self._h, C.byref(nt), C.byref(area)))
        return nt.value, area.value

    def triangles(self):
        nt = self.info()[0]
        p = np.empty((nt, 3, 3), np.float32)
        n = np.empty((nt, 3, 3), np.float32)
        check(load().rvh_mesh_triangles(self._h, _fp(p), _fp(n)))
        return p, n

    def sample_roots(self, n_roots, mode=MESH_ROOTS_REFERENCE, seed=8, normal_mode=ROOT_NORMAL_FIRST_CORNER):
        d = MeshRootsDesc(mode, n_roots, seed, normal_mode, 0)
        roots = np.empty((n_roots, 3), np.float32)
        normals = np.empty((n_roots, 3), np.float32)
        check(load().rvh_mesh_sample_roots(self._h, C.byref(d), _fp(roots), _fp(normals)))
        return roots, normals


def libc_rand_sequence(seed, n):
    out = np.empty(n, np.int32)
    check(load().rvh_libc_rand_sequence(seed, n, out.ctypes.data_as(C.POINTER(C.c_int32))))
    return out
