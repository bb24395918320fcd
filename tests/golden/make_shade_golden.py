"""Generate the shading fixture in tests/golden/ from the REFERENCE's own shaders.

Tessellates the reference-mode head after 60 frames (tests/golden/ref_head.npz,
96 strands of 10 points) with the oracle (12 isolines x 42 segments, the C
library's float sin in the hash, as the reference compiled here), builds the
light depth and deep opacity maps of all its vertices with the oracle, and
runs src/shaders/hair.frag and src/shaders/hairOpacity.frag (compiled as C++
against the reference's glm by oracle/build_ref_shade.py; needs the reference
checkout) on every 16th vertex's fragment inputs plus 64 fragments moved to
extreme light-space positions (outside the light frustum, behind the camera,
deep behind the first surface):

  shade_ref_head.npz   cameras (4, 16) glm's camera view, camera proj, light view,
                       light proj; depth (720, 1080); opacity (720, 1080, 4);
                       inputs (n, 24); rgba (n, 4) hair.frag's outColor;
                       layers (n, 4) hairOpacity.frag's outColor

Run: python tests/golden/make_shade_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import build_ref_shade  # noqa: E402
from oracle import oracle_ctypes as oracle  # noqa: E402

L, S, STRIDE, N_EXTREME = 12, 42, 16, 64


class _Desc:
    """The fields of a shading descriptor that the oracle reads."""

    def __init__(self, cams, w, h):
        self.camera_view, self.camera_proj, self.light_view, self.light_proj = [list(c) for c in cams]
        self.map_width, self.map_height = w, h


def reference_lib():
    path = build_ref_shade.build()
    if path is None:
        return None
    lib = C.CDLL(path)
    fp = C.POINTER(C.c_float)
    lib.ref_shade.argtypes = [C.c_int, fp, fp, fp, C.c_int, C.c_int, fp]
    lib.ref_opacity.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, fp]
    lib.ref_cameras.argtypes = [fp]
    for f in (lib.ref_shade, lib.ref_opacity, lib.ref_cameras):
        f.restype = C.c_int
    return lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def ref_cameras(lib):
    cams = np.zeros((4, 16), np.float32)
    assert lib.ref_cameras(_p(cams)) == 0
    return cams


def ref_shade(lib, inputs, depth, opacity):
    inp = np.ascontiguousarray(inputs, np.float32)
    h, w = depth.shape
    out = np.zeros((inp.shape[0], 4), np.float32)
    assert lib.ref_shade(inp.shape[0], _p(inp), _p(depth), _p(opacity), w, h, _p(out)) == 0
    return out


def ref_opacity(lib, inputs, depth):
    inp = np.ascontiguousarray(inputs, np.float32)
    h, w = depth.shape
    out = np.zeros((inp.shape[0], 4), np.float32)
    assert lib.ref_opacity(inp.shape[0], _p(inp), _p(depth), w, h, _p(out)) == 0
    return out


def fixture_inputs(cams):
    """(depth, opacity, inputs) of the fixture head from the oracle."""
    rec = np.ascontiguousarray(np.load(os.path.join(HERE, "ref_head.npz"))["state_60"], np.float32)
    verts, frames = oracle.tessellate(rec, 10, L, S, sin_mode=0, frames=True)
    desc = _Desc(cams, 1080, 720)
    depth, opacity = oracle.shade_maps(verts, desc)
    inputs = oracle.shade_vertex_inputs(verts, frames, 10, L, S, desc)[::STRIDE].copy()
    rng = np.random.default_rng(7)
    extreme = inputs[rng.choice(inputs.shape[0], N_EXTREME, replace=False)].copy()
    extreme[:, 17:20] = rng.uniform(-3.0, 3.0, (N_EXTREME, 3)).astype(np.float32)
    extreme[:, 20] = rng.choice([-1.0, 0.5, 1.0, 2.0], N_EXTREME).astype(np.float32)
    return depth, opacity, np.concatenate([inputs, extreme])


def main():
    lib = reference_lib()
    if lib is None:
        sys.exit("the reference checkout is not available")
    cams = ref_cameras(lib)
    depth, opacity, inputs = fixture_inputs(cams)
    rgba = ref_shade(lib, inputs, depth, opacity)
    layers = ref_opacity(lib, inputs, depth)
    np.savez_compressed(os.path.join(HERE, "shade_ref_head.npz"), cameras=cams, depth=depth, opacity=opacity,
                        inputs=inputs, rgba=rgba, layers=layers)
    print("wrote shade_ref_head.npz: %d fragments, %d covered texels, max layer %.3f"
          % (inputs.shape[0], int((depth < 1).sum()), float(opacity[..., :3].max())))


if __name__ == "__main__":
    main()
