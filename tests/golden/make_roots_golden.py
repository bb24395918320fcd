"""Generate the root-sampling fixtures in tests/golden/ from the REFERENCE's own code.

Writes a synthetic scalp mesh, scalp_mixed.obj (this project's own content: a
quad-dominant hemisphere cap with a 12-gon polar cap, a concave L-hexagon and
a concave star decagon, triangles; v, v/vt/vn, v//vn and negative indices),
then runs the reference's GeneratePointsOnMesh (src/Strand.cpp:26-146,
compiled with its vendored tiny_obj_loader and glm by oracle/build_ref_roots.py;
needs the reference checkout) on it:

  roots_scalp_mixed.npz   roots and normals for NUM_STRANDS = 4096 and 900
                          (srand(8), as the reference runs), and the
                          reference loader's triangle count.

Run: python tests/golden/make_roots_golden.py
"""
import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import build_ref_roots  # noqa: E402

OBJ = os.path.join(HERE, "scalp_mixed.obj")


def write_obj(path):
    lines = ["# synthetic scalp for root-sampling tests", "o scalp"]
    v, vn = [], []

    def vert(p, n):
        v.append(p)
        vn.append(n)
        return len(v)   # 1-based

    rings, seg = 6, 16
    idx = {}
    for i in range(1, rings + 1):
        th = 0.5 * math.pi * i / (rings + 1)
        for j in range(seg):
            ph = 2 * math.pi * j / seg
            n = (math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph))
            idx[i, j] = vert(n, n)
    for p in v:
        lines.append("v %.6f %.6f %.6f" % p)
    for n in vn:
        lines.append("vn %.6f %.6f %.6f" % n)
    lines.append("vt 0.5 0.5")
    # polar cap: one convex 12-gon through ring 1 (every other of 16 would skip; use 12 of them)
    cap = [idx[1, j] for j in range(0, seg) if j % 4 != 3]
    lines.append("f " + " ".join("%d//%d" % (k, k) for k in cap))
    lines.append("f %d//%d %d//%d %d//%d" % (idx[1, 2], idx[1, 2], idx[1, 3], idx[1, 3], idx[1, 4], idx[1, 4]))
    lines.append("s 1")
    for i in range(1, rings):
        for j in range(seg):
            a, b = idx[i, j], idx[i, (j + 1) % seg]
            c, d = idx[i + 1, (j + 1) % seg], idx[i + 1, j]
            if (i + j) % 5 == 0:   # split into two triangles, v/vt/vn form
                lines.append("f %d/1/%d %d/1/%d %d/1/%d" % (a, a, b, b, c, c))
                lines.append("f %d/1/%d %d/1/%d %d/1/%d" % (a, a, c, c, d, d))
            else:
                lines.append("f %d//%d %d//%d %d//%d %d//%d" % (a, a, b, b, c, c, d, d))
    # two concave flat polygons below the cap, given with negative (relative) indices
    lines.append("g flat")
    base = len(v)
    L = [(0, 0), (2, 0), (2, 1), (1, 1), (1, 2), (0, 2)]
    for (x, z) in L:
        lines.append("v %.6f %.6f %.6f" % (1.5 + 0.1 * x, 0.05, 0.1 * z))
    lines.append("vn 0 1 0")
    lines.append("f " + " ".join("%d//-1" % (-(len(L) - k)) for k in range(len(L))))
    star = []
    for k in range(10):
        r = 0.25 if k % 2 == 0 else 0.1
        a = 2 * math.pi * k / 10
        star.append((-1.5 + r * math.cos(a), 0.05, r * math.sin(a)))
    for p in star:
        lines.append("v %.6f %.6f %.6f" % p)
    lines.append("f " + " ".join("%d//-1" % (base + len(L) + 1 + k) for k in range(10)))
    open(path, "w").write("\n".join(lines) + "\n")


def ref_roots(lib, n):
    roots = np.zeros((n, 3), np.float32)
    normals = np.zeros((n, 3), np.float32)
    r = lib.ref_roots(OBJ.encode(), n, roots.ctypes.data, normals.ctypes.data)
    assert r == n
    return roots, normals


def main():
    write_obj(OBJ)
    path = build_ref_roots.build()
    if path is None:
        sys.exit("the reference checkout is not available")
    lib = C.CDLL(path)
    lib.ref_roots.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p]
    lib.ref_roots.restype = C.c_int
    out = {}
    for n in (4096, 900):
        r, q = ref_roots(lib, n)
        out["roots_%d" % n] = r
        out["normals_%d" % n] = q
    np.savez_compressed(os.path.join(HERE, "roots_scalp_mixed.npz"), **out)
    print("wrote", OBJ, "and roots_scalp_mixed.npz")


if __name__ == "__main__":
    main()
