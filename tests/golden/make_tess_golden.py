"""Generate the tessellation fixture in tests/golden/ from the REFERENCE's own shader.

Runs src/shaders/hair.tese (compiled as C++ against the reference's glm by
oracle/build_ref_tess.py; needs the reference checkout) on the first 8 strands
of the reference-mode head after 60 frames (tests/golden/ref_head.npz,
10 points per strand) with the tessellation levels of src/shaders/hair.tesc
(12 isolines x 42 segments), and records gl_Position.xyz + out_strandWidth and
the {out_u, out_v, out_w} frame of every vertex:

  tess_ref_head.npz   records (8, 30, 4), vertices (8, 12, 43, 4), frames (8, 12, 43, 9)

The shader reads past the strand at v = 1 (k = 42); those entries are kept
but not meaningful.

Run: python tests/golden/make_tess_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import build_ref_tess  # noqa: E402

L, S, NS = 12, 42, 8


def main():
    path = build_ref_tess.build()
    if path is None:
        sys.exit("the reference checkout is not available")
    lib = C.CDLL(path)
    lib.ref_tess.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lib.ref_tess.restype = C.c_int
    rec = np.ascontiguousarray(np.load(os.path.join(HERE, "ref_head.npz"))["state_60"][:NS], np.float32)
    out = np.zeros((NS, L, S + 1, 4), np.float32)
    fr = np.zeros((NS, L, S + 1, 9), np.float32)
    assert lib.ref_tess(rec.ctypes.data, NS, L, S, out.ctypes.data, fr.ctypes.data) == 0
    np.savez_compressed(os.path.join(HERE, "tess_ref_head.npz"), records=rec, vertices=out, frames=fr)
    print("wrote tess_ref_head.npz")


if __name__ == "__main__":
    main()
