"""ctypes mirrors of include/rvh_types.h (layouts checked by tests/test_abi.py)."""
import ctypes as C

import numpy as np

MAX_COLLIDERS = 8
MAX_POINTS = 32
MIN_POINTS = 2

OK = 0
ERR_INVALID_ARG = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_BUDGET = 4
ERR_TIMEOUT = 5
ERR_STATE = 6
ERR_UNSUPPORTED = 7
ERR_NO_DEVICE = 8

COLLIDER_SPHERE = 0
COLLIDER_ELLIPSOID = 1

MEM_HOST = 0
MEM_DEVICE = 1
MEM_DEVICE_BORROWED = 2


class Collider(C.Structure):
    """struct Collider (src/Scene.h:23-27): transform, inv, invTrans (column-major) + kind."""
    _fields_ = [("transform", C.c_float * 16), ("inv", C.c_float * 16), ("inv_trans", C.c_float * 16),
                ("kind", C.c_int32), ("radius", C.c_float), ("attach_to_head", C.c_int32),
                ("reserved", C.c_int32)]

    def matrices(self):
        return (np.array(self.transform, np.float32).reshape(4, 4).T,
                np.array(self.inv, np.float32).reshape(4, 4).T,
                np.array(self.inv_trans, np.float32).reshape(4, 4).T)


class SimParams(C.Structure):
    _fields_ = [("gravity", C.c_float * 3), ("damping", C.c_float), ("dftl_damping", C.c_float),
                ("vmax", C.c_float), ("k_penalty", C.c_float), ("friction", C.c_float),
                ("repulsion", C.c_float), ("grid_scale", C.c_float), ("grid_enabled", C.c_int32),
                ("grid_wrap32", C.c_int32), ("grid_origin", C.c_float * 3), ("grid_h", C.c_float),
                ("grid_dims", C.c_int32 * 3), ("reserved", C.c_int32)]


class Frame(C.Structure):
    """struct Time (src/Scene.h:16-19) + wind."""
    _fields_ = [("dt", C.c_float), ("t", C.c_float), ("wind", C.c_float * 3), ("reserved", C.c_int32)]


class DrawIndirect(C.Structure):
    """struct StrandDrawIndirect (src/Strand.h:53-58)."""
    _fields_ = [("vertex_count", C.c_uint32), ("instance_count", C.c_uint32),
                ("first_vertex", C.c_uint32), ("first_instance", C.c_uint32)]


class HeadDesc(C.Structure):
    """rvh_head_desc (include/rvh_scene.h): a seeded synthetic head."""
    _fields_ = [("seed", C.c_uint64), ("n_strands", C.c_int32), ("n_points", C.c_int32),
                ("head_radius", C.c_float), ("head_center", C.c_float * 3), ("root_sampling", C.c_int32),
                ("sort_roots", C.c_int32), ("length_min", C.c_float), ("length_max", C.c_float),
                ("head_collider", C.c_int32), ("n_ellipsoids", C.c_int32), ("axis_min", C.c_float),
                ("axis_max", C.c_float), ("grid_res", C.c_int32), ("friction", C.c_float),
                ("repulsion", C.c_float), ("dftl_damping", C.c_float)]


class WindDesc(C.Structure):
    """rvh_wind_desc (include/rvh_scene.h): closed-form wind plus seeded gusts."""
    _fields_ = [("amplitude", C.c_float), ("omega", C.c_float), ("dir", C.c_float * 3), ("gust_sigma", C.c_float),
                ("seed", C.c_uint64)]


def head_desc(**kw):
    """A HeadDesc with head radius 1 and the reference's DFTL damping unless given."""
    d = HeadDesc()
    d.head_radius = 1.0
    d.dftl_damping = 0.0
    for k, v in kw.items():
        if k == "head_center":
            d.head_center[:] = v
        else:
            setattr(d, k, v)
    return d


def reference_params():
    """The constants hard-coded in src/shaders/compute.comp (lines cited in rvh_types.h)."""
    p = SimParams()
    p.gravity[:] = (0.0, -9.8, 0.0)
    p.damping = 0.998
    p.dftl_damping = 0.998
    p.vmax = 10.0
    p.k_penalty = 1900.0
    p.friction = 0.08
    p.repulsion = 0.0
    p.grid_scale = 1000000.0
    p.grid_enabled = 1
    p.grid_wrap32 = 1
    p.grid_origin[:] = (-3.0, -2.0, -5.0)
    p.grid_h = np.float32(7.0) / np.float32(64.0)
    p.grid_dims[:] = (64, 64, 64)
    return p


def frame(dt, t=0.0, wind=(0.0, 0.0, 0.0)):
    f = Frame()
    f.dt = dt
    f.t = t
    f.wind[:] = wind
    return f


def frames_array(frames):
    arr = (Frame * len(frames))()
    for i, f in enumerate(frames):
        arr[i] = f
    return arr


def colliders_array(rows):
    """rows: list (steps) of lists of Collider -> flat ctypes array (steps*ncol)."""
    flat = [c for row in rows for c in row]
    arr = (Collider * max(1, len(flat)))()
    for i, c in enumerate(flat):
        arr[i] = c
    return arr


def collider_from_mats(transform, inv, inv_trans, kind=COLLIDER_ELLIPSOID, radius=1.0):
    c = Collider()
    c.transform[:] = np.asarray(transform, np.float32).T.reshape(-1).tolist()
    c.inv[:] = np.asarray(inv, np.float32).T.reshape(-1).tolist()
    c.inv_trans[:] = np.asarray(inv_trans, np.float32).T.reshape(-1).tolist()
    c.kind = kind
    c.radius = radius
    return c


def collider_from_flat48(flat48, kind=COLLIDER_ELLIPSOID, radius=1.0):
    c = Collider()
    f = np.asarray(flat48, np.float32).reshape(-1)
    c.transform[:] = f[0:16].tolist()
    c.inv[:] = f[16:32].tolist()
    c.inv_trans[:] = f[32:48].tolist()
    c.kind = kind
    c.radius = radius
    return c


def sphere_collider(center, radius):
    """A sphere collider: centre in transform[3].xyz (the reference reads colliders[0] this way)."""
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = center
    inv = np.eye(4, dtype=np.float32)
    inv[:3, 3] = -np.asarray(center, np.float32)
    return collider_from_mats(m, inv, inv.T, COLLIDER_SPHERE, radius)
