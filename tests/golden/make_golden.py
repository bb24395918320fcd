"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own code.

Runs src/shaders/compute.comp (compiled as C++ against the reference's glm by
oracle/build_ref.py; needs the reference checkout, named by $RVH_REFERENCE_DIR)
on seeded reference-mode scenes, and records inputs and outputs:

  ref_head.npz   96 strands x 10 points rooted on the reference's head
                 ellipsoid, the six colliders of src/main.cpp:229-237 built by
                 glm as Scene.h:28-39 does, the sphere moved every frame with
                 Scene::translateSphere (Scene.cpp:110-120); 60 frames of
                 dt = 1/60; states after frames 1, 10, 60 and the last grid.
  ref_dense.npz  256 strands rooted in one small patch, so grid cells exceed
                 the int32 range and wrap as the shader's atomicAdd does;
                 2 frames; states and the last grid.
  colliders.npz  glm's Collider matrices for the main.cpp colliders and a
                 translated copy (pins rvh_collider_from_trs / _translate).

Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import oracle_ctypes as O  # noqa: E402

# trans, rot (deg), scale of the six colliders in src/main.cpp:229-237 (sphere first)
MAIN_COLLIDERS = [
    ((2.0, 0.0, 1.0), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)),
    ((0.0, 2.64, 0.08), (-38.270, 0.0, 0.0), (0.817, 1.158, 1.01)),
    ((0.0, 1.35, -0.288), (18.301, 0.0, 0.0), (0.457, 1.0, 0.538)),
    ((0.0, -0.380, -0.116), (-17.260, 0.0, 0.0), (1.078, 1.683, 0.974)),
    ((-0.698, 0.087, -0.36), (-20.254, 13.144, 34.5), (0.721, 1.0, 0.724)),
    ((0.698, 0.087, -0.36), (-20.254, 13.144, -34.5), (0.721, 1.0, 0.724)),
]
N = 10            # NUM_CURVE_POINTS, compute.comp:5
LENGTH = 2.5      # compute.comp:139
DT = np.float32(1.0 / 60.0)


def reference_strands(roots, normals):
    """Hair::Hair's initial strands (Strand.cpp:157-175), written out here."""
    ns = roots.shape[0]
    st = np.zeros((ns, 3 * N, 4), np.float32)
    seg = np.float32(np.float32(LENGTH) / (np.float32(N) - np.float32(1.0)))
    for s in range(ns):
        p = roots[s].astype(np.float32).copy()
        d = normals[s].astype(np.float32).copy()
        d[2] -= np.float32(2.0)
        d[1] += np.float32(5.0)
        d[0] += np.float32(0.05)
        for j in range(N):
            st[s, j, :3] = p
            st[s, j, 3] = 1.0
            st[s, N + j] = (0.0, 0.0, -1.0, 0.0)
            p = (p + seg * d).astype(np.float32)
    return st


def head_roots(cols48, ns, rng, spread=1.0):
    head = cols48[1]
    M = head[:16].reshape(4, 4).T.astype(np.float64)
    IT = head[32:48].reshape(4, 4).T.astype(np.float64)
    u = rng.normal(size=(ns, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    u[:, 1] = np.abs(u[:, 1]) + 0.3 / spread
    if spread < 1.0:
        u[:, 0] *= spread
        u[:, 2] *= spread
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    roots = (M @ np.c_[u * 1.02, np.ones(ns)].T).T[:, :3]
    nrm = (IT @ np.c_[u, np.zeros(ns)].T).T[:, :3]
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return roots.astype(np.float32), nrm.astype(np.float32)


def sparse_grid(g):
    nz = np.nonzero(np.any(g != 0, axis=1))[0].astype(np.int32)
    return nz, g[nz]


def run_case(strands, cols48, steps, move, snaps):
    cs = np.repeat(cols48[None], steps, 0).copy()
    for k in range(1, steps):
        cs[k, 0] = O.ref_translate(cs[k - 1, 0], move)
    times = np.stack([np.full(steps, DT), (np.arange(1, steps + 1) * DT).astype(np.float32)], 1).astype(np.float32)
    out = {}
    st = strands.copy()
    done = 0
    grid = None
    for s in sorted(snaps):
        grid, draw = O.ref_run(st, cs[done:s], times[done:s], want_grid=True)
        done = s
        out["state_%d" % s] = st.copy()
    idx, val = sparse_grid(grid)
    out.update(colliders=cs, times=times, grid_index=idx, grid_value=val, draw=draw)
    return out


def main():
    if not O.ref_available():
        raise SystemExit("the reference checkout is not available; fixtures cannot be regenerated")
    cols48 = np.stack([O.ref_collider(*c) for c in MAIN_COLLIDERS]).astype(np.float32)

    rng = np.random.default_rng(20190101)
    roots, nrm = head_roots(cols48, 96, rng)
    init = reference_strands(roots, nrm)
    res = run_case(init, cols48, 60, (-0.03, 0.04, 0.0), [1, 10, 60])
    np.savez_compressed(os.path.join(HERE, "ref_head.npz"), init=init, n_points=N, **res)

    rng = np.random.default_rng(7)
    roots, nrm = head_roots(cols48, 256, rng, spread=0.02)
    init = reference_strands(roots, nrm)
    res = run_case(init, cols48, 2, (0.0, 0.0, 0.0), [1, 2])
    np.savez_compressed(os.path.join(HERE, "ref_dense.npz"), init=init, n_points=N, **res)

    moved = O.ref_translate(cols48[0], (0.25, -0.5, 1.0))
    np.savez_compressed(os.path.join(HERE, "colliders.npz"), specs=np.array(MAIN_COLLIDERS, np.float32),
                        mats=cols48, sphere_moved=moved, move=np.array((0.25, -0.5, 1.0), np.float32))
    for f in ("ref_head.npz", "ref_dense.npz", "colliders.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
