"""Scalp meshes and hair-root sampling (src/Strand.cpp:26-146), CPU only.

The reference-mode sampler must give the bits of the reference's own
GeneratePointsOnMesh: against the committed fixture (made by running the
reference's code, tests/golden/make_roots_golden.py) and, where the reference
checkout exists, live against the compiled reference on its own meshes.
"""
import ctypes as C
import ctypes.util
import os

import numpy as np
import pytest

from conftest import ROOT
from rvh import api
from rvh import types as T
from rvh._lib import RvhError

GOLDEN = os.path.join(ROOT, "tests", "golden")
OBJ = os.path.join(GOLDEN, "scalp_mixed.obj")


def _libc():
    name = ctypes.util.find_library("c")
    if not name:
        pytest.skip("no C library found")
    lib = C.CDLL(name)
    if not hasattr(lib, "gnu_get_libc_version"):
        pytest.skip("rand() of this C library is not glibc's")
    return lib


@pytest.mark.parametrize("seed", [8, 0, 1, 12345, 2**31 + 5, 2**32 - 1])
def test_rand_restatement_matches_glibc(librvh, seed):
    libc = _libc()
    libc.srand(C.c_uint(seed))
    want = np.array([libc.rand() for _ in range(3000)], np.int32)
    assert np.array_equal(api.libc_rand_sequence(seed, 3000), want)


@pytest.mark.parametrize("n", [4096, 900])
def test_reference_roots_match_golden(librvh, n):
    g = np.load(os.path.join(GOLDEN, "roots_scalp_mixed.npz"))
    m = api.Mesh.load_obj(OBJ)
    roots, normals = m.sample_roots(n, mode=api.MESH_ROOTS_REFERENCE, seed=8)
    assert np.array_equal(roots.view(np.uint32), g["roots_%d" % n].view(np.uint32))
    assert np.array_equal(normals.view(np.uint32), g["normals_%d" % n].view(np.uint32))


def _ref_lib():
    from oracle import build_ref_roots
    if not build_ref_roots.available():
        pytest.skip("reference checkout not present")
    lib = C.CDLL(build_ref_roots.build())
    lib.ref_roots.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p]
    lib.ref_roots.restype = C.c_int
    return lib, build_ref_roots.reference_dir()


@pytest.mark.parametrize("obj", ["mannequin_segment.obj", "mannequin_segment2.obj", "hemisphere.obj",
                                 "collisionTest.obj"])
def test_reference_roots_match_compiled_reference_live(librvh, obj):
    lib, ref = _ref_lib()
    path = os.path.join(ref, "src", "models", obj)
    if not os.path.isfile(path):
        pytest.skip("mesh not present")
    n = 900   # NUM_STRANDS of the reference's own build
    rr = np.zeros((n, 3), np.float32)
    rn = np.zeros((n, 3), np.float32)
    assert lib.ref_roots(path.encode(), n, rr.ctypes.data, rn.ctypes.data) == n
    roots, normals = api.Mesh.load_obj(path).sample_roots(n)
    assert np.array_equal(roots.view(np.uint32), rr.view(np.uint32))
    assert np.array_equal(normals.view(np.uint32), rn.view(np.uint32))


def _poly_area(p):
    """Area of a planar polygon (3-D vertices) by the shoelace vector sum."""
    s = np.zeros(3)
    for k in range(len(p)):
        s += np.cross(p[k], p[(k + 1) % len(p)])
    return 0.5 * np.linalg.norm(s)


def test_concave_polygons_are_covered_exactly(librvh, tmp_path):
    # an L hexagon and a star decagon: the triangles tile each polygon
    L = np.array([(0, 0, 0), (2, 0, 0), (2, 0, 1), (1, 0, 1), (1, 0, 2), (0, 0, 2)], float)
    ang = 2 * np.pi * np.arange(10) / 10
    r = np.where(np.arange(10) % 2 == 0, 1.0, 0.4)
    star = np.stack([r * np.cos(ang), np.zeros(10), r * np.sin(ang)], 1)
    for poly in (L, star):
        path = tmp_path / "p.obj"
        txt = "".join("v %r %r %r\n" % tuple(float(c) for c in q) for q in poly) + "vn 0 1 0\n"
        txt += "f " + " ".join("%d//1" % (k + 1) for k in range(len(poly))) + "\n"
        path.write_text(txt)
        m = api.Mesh.load_obj(str(path))
        nt, area = m.info()
        assert nt == len(poly) - 2
        assert area == pytest.approx(_poly_area(poly), rel=1e-6)
        pos, nrm = m.triangles()
        # every triangle keeps the polygon's orientation (no flipped ear)
        for t in pos.astype(float):
            assert np.cross(t[1] - t[0], t[2] - t[0])[1] <= 1e-9


def test_quad_split_is_the_loaders_fan(librvh, tmp_path):
    path = tmp_path / "q.obj"
    path.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1 4//1\n")
    pos, _ = api.Mesh.load_obj(str(path)).triangles()
    assert np.array_equal(pos[0], np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0]], np.float32))
    assert np.array_equal(pos[1], np.array([[0, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32))


def test_negative_indices_and_missing_normals(librvh, tmp_path):
    path = tmp_path / "n.obj"
    path.write_text("v 0 0 0\nv 2 0 0\nv 0 0 2\nf -3 -1 -2\n")
    m = api.Mesh.load_obj(str(path))
    pos, nrm = m.triangles()
    assert np.array_equal(pos[0], np.array([[0, 0, 0], [0, 0, 2], [2, 0, 0]], np.float32))
    # no normals in the file: the triangle's geometric normal
    assert np.allclose(nrm[0], [[0, 1, 0]] * 3)


@pytest.mark.parametrize("text", ["v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 7\n",
                                  "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//5\n"])
def test_bad_indices_are_errors(librvh, tmp_path, text):
    path = tmp_path / "bad.obj"
    path.write_text(text)
    with pytest.raises(RvhError) as e:
        api.Mesh.load_obj(str(path))
    assert e.value.status == T.ERR_INVALID_ARG


def test_missing_file_is_an_error(librvh, tmp_path):
    with pytest.raises(RvhError):
        api.Mesh.load_obj(str(tmp_path / "absent.obj"))


def _two_triangles():
    # areas 1 and 9 in the y = 0 plane
    p = np.array([[[0, 0, 0], [0, 0, 2], [1, 0, 0]], [[5, 0, 0], [5, 0, 6], [8, 0, 0]]], np.float32)
    n = np.tile(np.array([0, 1, 0], np.float32), (2, 3, 1))
    return api.Mesh.from_triangles(p, n), p


def test_area_uniform_roots_follow_triangle_area(librvh):
    m, p = _two_triangles()
    assert m.info()[1] == pytest.approx(10.0)
    n = 40000
    roots, normals = m.sample_roots(n, mode=api.MESH_ROOTS_AREA, seed=3)
    big = roots[:, 0] >= 4.0
    frac = big.mean()
    assert abs(frac - 0.9) < 4 * np.sqrt(0.09 / n)       # 4 sigma of a binomial
    # every root lies in its triangle: barycentric coordinates in [0, 1]
    for t, sel in ((0, ~big), (1, big)):
        a, b, c = p[t].astype(float)
        M = np.stack([b - a, c - a], 1)[[0, 2]]
        uv = np.linalg.solve(M, (roots[sel].astype(float) - a)[:, [0, 2]].T).T
        assert (uv >= -1e-6).all() and (uv.sum(1) <= 1 + 1e-6).all()
    # uniform inside a triangle: the mean is the centroid
    assert np.allclose(roots[big].mean(0), p[1].mean(0), atol=0.05)
    assert np.allclose(normals, [0, 1, 0])
    again, _ = m.sample_roots(n, mode=api.MESH_ROOTS_AREA, seed=3)
    assert np.array_equal(roots, again)
    other, _ = m.sample_roots(n, mode=api.MESH_ROOTS_AREA, seed=4)
    assert not np.array_equal(roots, other)


def test_reference_mode_is_triangle_uniform(librvh):
    m, _ = _two_triangles()
    roots, _ = m.sample_roots(40000, mode=api.MESH_ROOTS_REFERENCE, seed=8)
    assert abs((roots[:, 0] >= 4.0).mean() - 0.5) < 0.02   # the reference ignores triangle area


def test_interpolated_normals_are_unit(librvh):
    m = api.Mesh.load_obj(OBJ)
    _, nrm = m.sample_roots(2000, mode=api.MESH_ROOTS_AREA, seed=1, normal_mode=api.ROOT_NORMAL_INTERPOLATED)
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-6)


def test_roots_feed_the_reference_strand_builder(librvh):
    m = api.Mesh.load_obj(OBJ)
    roots, normals = m.sample_roots(64)
    rec = api.init_strands_reference(roots, normals, 10, 2.5 / 9.0)
    assert np.array_equal(rec[:, 0, :3], roots)
    d = normals.astype(np.float32) + np.array([0.05, 5.0, -2.0], np.float32)
    assert np.allclose(rec[:, 1, :3], roots + np.float32(2.5 / 9.0) * d, atol=1e-6)
