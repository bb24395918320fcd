"""Hair shading: the shadow, opacity and hair passes (src/Renderer.cpp,
src/shaders/hairOpacity.frag, src/shaders/hair.frag).

CPU: the oracle's restatement against the reference's own fragment shaders,
compiled as C++ with its glm (tests/golden/shade_ref_head.npz, made by
tests/golden/make_shade_golden.py; and live where the reference checkout
exists), bit for bit; the library's reference cameras against glm's.
GPU: rvh_shade_fragments against the reference's outputs, and
rvh_asset_shade / rvh_render_image against the oracle: the light depth and
opacity maps and the camera image's depth test bit for bit, the colours within
COLOR_TOL — the only difference is CUDA's acos, sin, cos, exp and pow against
the C library's (a few float ulps each; the brightness hash uses a correctly
rounded sin on both sides).
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT
from rvh import api

GOLDEN = os.path.join(ROOT, "tests", "golden")
COLOR_TOL = 1e-4   # absolute, per colour channel in [0, 1]


def _fixture():
    return np.load(os.path.join(GOLDEN, "shade_ref_head.npz"))


def _same_bits(a, b):
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


class _Desc:
    def __init__(self, cams, w, h):
        self.camera_view, self.camera_proj, self.light_view, self.light_proj = [list(c) for c in cams]
        self.map_width, self.map_height = w, h


def test_oracle_matches_reference_fragment_shader_golden(oracle):
    g = _fixture()
    out = oracle.shade_fragments(g["inputs"], g["depth"], g["opacity"], sin_mode=0)
    assert _same_bits(out, g["rgba"])
    # the fixture covers lit and shadowed fragments, all layers the head reaches and the clipped ones
    assert (g["rgba"][:, :3].std(0) > 0.01).all()


def test_oracle_matches_reference_opacity_shader_golden(oracle):
    g = _fixture()
    out = oracle.opacity_fragments(g["inputs"], g["depth"])
    assert _same_bits(out, g["layers"])
    assert (g["layers"][:, 0] > 0).any() and (g["layers"][:, 2] > 0).any() and (g["layers"][:, 2] == 0).any()


def test_correctly_rounded_hash_agrees_on_the_reference_isolines(oracle):
    g = _fixture()
    out = oracle.shade_fragments(g["inputs"], g["depth"], g["opacity"], sin_mode=1)
    assert _same_bits(out, g["rgba"])


def test_reference_cameras_match_glm(librvh):
    g = _fixture()
    d = api.shade_desc_reference()
    for k, name in enumerate(("camera_view", "camera_proj", "light_view", "light_proj")):
        assert _same_bits(np.array(list(getattr(d, name)), np.float32), g["cameras"][k]), name
    assert (d.map_width, d.map_height) == (1080, 720)


def test_oracle_maps_properties(oracle):
    g = _fixture()
    depth, layers = g["depth"], g["opacity"][..., :3]
    assert ((depth > 0) & (depth <= 1)).all()
    allowed = np.array([0, 77, 154, 231, 255], np.float32) / np.float32(255)
    assert np.isin(layers, allowed).all()
    assert (layers[..., 0] <= layers[..., 1]).all() and (layers[..., 1] <= layers[..., 2]).all()
    assert (g["opacity"][..., 3] == 0).all()


def test_oracle_image_keeps_the_nearest_vertex(oracle):
    desc = _Desc(_fixture()["cameras"], 64, 48)
    verts = np.array([[0.0, 1.0, 0.0, 1], [0.0, 1.0, 0.5, 1], [0.0, 1.0, -0.5, 1], [50.0, 1.0, 0.0, 1]], np.float32)
    colors = np.array([[1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 1], [1, 1, 1, 1]], np.float32)
    img = oracle.render_image(verts, colors, desc, 64, 48)
    lit = img.reshape(-1, 4)[(img.reshape(-1, 4) != 0).any(1)]
    assert lit.shape[0] == 1 and np.array_equal(lit[0], colors[1])   # the one nearest the camera at z = 10


def test_oracle_matches_reference_shaders_live(oracle):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_shade_golden as mk
    lib = mk.reference_lib()
    if lib is None:
        pytest.skip("reference checkout not present")
    cams = mk.ref_cameras(lib)
    rec = np.ascontiguousarray(np.load(os.path.join(GOLDEN, "ref_head.npz"))["state_10"], np.float32)
    verts, frames = oracle.tessellate(rec, 10, 12, 42, sin_mode=0, frames=True)
    desc = _Desc(cams, 540, 360)
    depth, opacity = oracle.shade_maps(verts, desc)
    inputs = oracle.shade_vertex_inputs(verts, frames, 10, 12, 42, desc)[::3]
    assert _same_bits(oracle.shade_fragments(inputs, depth, opacity, sin_mode=0), mk.ref_shade(lib, inputs, depth,
                                                                                              opacity))
    assert _same_bits(oracle.opacity_fragments(inputs, depth), mk.ref_opacity(lib, inputs, depth))


# ---- GPU ----------------------------------------------------------------------------

def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _colors_close(got, want):
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    err = np.abs(got - want)[~nan]
    print("colour max |diff| %.3g" % (err.max() if err.size else 0.0))
    assert err.size == 0 or err.max() <= COLOR_TOL


@pytest.mark.gpu
def test_gpu_fragments_match_reference_golden(gpu_ctx, oracle):
    import torch
    g = _fixture()
    inp, dep, opa = _dev(g["inputs"]), _dev(g["depth"]), _dev(g["opacity"])
    n = g["inputs"].shape[0]
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    h, w = g["depth"].shape
    api.shade_fragments(gpu_ctx, n, inp.data_ptr(), dep.data_ptr(), opa.data_ptr(), w, h, out.data_ptr())
    gpu_ctx.synchronize()
    got = out.cpu().numpy()
    _colors_close(got, g["rgba"])
    assert (got[:, 3] == 0.75).all()


def _shade_on_gpu(ctx, a, ns, n, td, sd):
    import torch
    per = td.n_lines * (td.n_segments + 1)
    vert = torch.zeros((ns * per * 4,), dtype=torch.float32, device="cuda")
    fr = torch.zeros((ns * (n - 1) * 12,), dtype=torch.float32, device="cuda")
    texels = sd.map_width * sd.map_height
    depth = torch.full((texels,), -7.0, dtype=torch.float32, device="cuda")    # every texel is written
    opac = torch.full((texels * 4,), -7.0, dtype=torch.float32, device="cuda")
    col = torch.zeros((ns * per * 4,), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    a.tessellate(vert.data_ptr(), fr.data_ptr(), desc=td)
    a.shade(vert.data_ptr(), fr.data_ptr(), depth.data_ptr(), opac.data_ptr(), col.data_ptr(), tess_desc=td,
            shade_desc=sd)
    ctx.synchronize()
    return (vert.cpu().numpy().reshape(ns, td.n_lines, td.n_segments + 1, 4),
            fr.cpu().numpy().reshape(ns, n - 1, 3, 4),
            depth.cpu().numpy().reshape(sd.map_height, sd.map_width),
            opac.cpu().numpy().reshape(sd.map_height, sd.map_width, 4),
            col.cpu().numpy().reshape(-1, 4), (vert, col))


def _head(ctx, seed, n, ns=400):
    rec, rest, p, cols = api.generate_head(seed=seed, n_strands=ns, n_points=n, root_sampling=0, sort_roots=1,
                                           length_min=0.3, length_max=0.9, head_collider=1, n_ellipsoids=1,
                                           axis_min=0.2, axis_max=0.4, grid_res=0, friction=0.0, repulsion=0.0,
                                           dftl_damping=0.9)
    a = api.Asset(ctx, rec, n, rest=rest)
    a.set_params(p)
    a.set_colliders(cols)
    for k in range(3):
        a.step(api.T.frame(np.float32(1.0 / 60.0), np.float32((k + 1) / 60.0)))
    return a, rec.shape[0]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [api.SHADE_MAPS_QUADS, api.SHADE_MAPS_VERTICES])
@pytest.mark.parametrize("n,lines,segs,mw,mh", [(10, 12, 42, 1080, 720), (16, 5, 17, 270, 180), (32, 8, 64, 333, 97),
                                                (16, 12, 42, 8, 6), (16, 12, 42, 2, 1)])   # tiny maps: layers saturate
def test_gpu_asset_shade_matches_oracle(gpu_ctx, oracle, n, lines, segs, mw, mh, mode):
    a, ns = _head(gpu_ctx, seed=n + lines, n=n)
    td = api.tess_desc_reference(n_lines=lines, n_segments=segs)
    sd = api.shade_desc_reference(map_width=mw, map_height=mh, map_mode=mode)
    verts, frames, depth, opac, col, _ = _shade_on_gpu(gpu_ctx, a, ns, n, td, sd)
    want_depth, want_opac = oracle.shade_maps(verts, sd)
    assert _same_bits(depth, want_depth)
    assert _same_bits(opac, want_opac)
    if mw * mh >= 1000 or mode == api.SHADE_MAPS_VERTICES:   # a tiny map may catch no quad's pixel centre
        need = 100 if mw * mh >= 1000 else 1
        assert (depth < 1).sum() >= need and (opac[..., 0] > 0).sum() >= need
    if mw * mh <= 48 and mode == api.SHADE_MAPS_VERTICES:   # thousands of vertices per texel: layers saturate
        cov = depth < 1
        assert (opac[..., 2][cov] == 1.0).all()
    inputs = oracle.shade_vertex_inputs(verts, frames, n, lines, segs, sd)
    want = oracle.shade_fragments(inputs, want_depth, want_opac, sin_mode=1)
    _colors_close(col, want)
    a.close()


@pytest.mark.gpu
def test_gpu_render_image_matches_oracle(gpu_ctx, oracle):
    import torch
    a, ns = _head(gpu_ctx, seed=3, n=10)
    td, sd = api.tess_desc_reference(), api.shade_desc_reference()
    verts, _, _, _, col, (vert_d, col_d) = _shade_on_gpu(gpu_ctx, a, ns, 10, td, sd)
    w, h = 1080, 720
    img = torch.full((w * h * 4,), -7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    nv = verts.reshape(-1, 4).shape[0]
    api.render_image(gpu_ctx, nv, vert_d.data_ptr(), col_d.data_ptr(), w, h, img.data_ptr(), shade_desc=sd)
    gpu_ctx.synchronize()
    got = img.cpu().numpy().reshape(h, w, 4)
    want = oracle.render_image(verts, col, sd, w, h)
    assert _same_bits(got, want)
    assert (got[..., 3] == 0.75).sum() > 1000
    a.close()


def test_oracle_raster_image_basics(oracle):
    """The oracle's rasterised image: covered pixels carry hair.frag's alpha and a
    valid segment id, the rest stay empty."""
    from oracle.oracle_ctypes import render_hair
    rec, rest, p, cols = api.generate_head(seed=9, n_strands=40, n_points=10, root_sampling=0, sort_roots=1,
                                           length_min=0.4, length_max=0.8, head_collider=1, n_ellipsoids=0,
                                           grid_res=0, friction=0.0, repulsion=0.0, dftl_damping=0.9)
    v, fr = oracle.tessellate(rec, 10, 12, 42, sin_mode=1, frames=True)
    sd = api.shade_desc_reference(map_width=270, map_height=180, image_mode=api.IMAGE_NEAREST)
    d, op = oracle.shade_maps(v, sd)
    img, ids = render_hair(v, fr, 10, 12, 42, sd, d, op, 540, 360)
    hit = ids != 0xffffffff
    assert hit.sum() > 500
    assert (img[hit][:, 3] == 0.75).all() and (img[~hit] == 0).all()
    assert ids[hit].max() < 40 * 12 * 42
    # the reference pipeline's blending: the same nearest fragment per pixel; a pixel
    # with one fragment is 0.75 c + 0.25 clear, an empty one keeps the clear colour
    sd.image_mode = api.IMAGE_BLEND
    img_b, ids_b = render_hair(v, fr, 10, 12, 42, sd, d, op, 540, 360)
    assert np.array_equal(ids_b, ids)
    clear = oracle.CLEAR_RGBA
    assert (img_b[~hit] == clear).all() and (img_b[..., 3] == 1.0).all()
    one = hit & (np.abs(img_b[..., :3] - (0.75 * img[..., :3] + 0.25 * clear[:3])).max(axis=-1) < 1e-6)
    assert one.sum() > 0.3 * hit.sum()   # most pixels are covered by one fragment


def test_oracle_blending_follows_primitive_order(oracle):
    """Two quads on one line of sight: drawn far then near, both fragments blend
    (the near one passes the LESS test after the far one); drawn near then far,
    only the near one does.  The segment drawn first is the first in memory."""
    from oracle.oracle_ctypes import render_hair
    n, L, S = 2, 1, 1
    frames = np.zeros((2, n - 1, 3, 4), np.float32)
    frames[:, 0, 0, :3] = (1, 0, 0)
    frames[:, 0, 1, :3] = (0, 1, 0)
    frames[:, 0, 2, :3] = (0, 0, 1)
    near = [[0.0, 0.5, 2.0, 0.3], [0.0, 1.5, 2.0, 0.3]]      # vertical: the quads widen along x
    far = [[0.0, 0.5, -2.0, 0.3], [0.0, 1.5, -2.0, 0.3]]
    sd = api.shade_desc_reference(map_width=64, map_height=64, image_mode=api.IMAGE_BLEND)
    W, H = 360, 240
    out = {}
    for name, order in (("far_first", [far, near]), ("near_first", [near, far])):
        verts = np.array([[o] for o in order], np.float32)   # (2, L, S+1, 4)
        d, op = oracle.shade_maps(verts, sd)
        out[name] = render_hair(verts, frames, n, L, S, sd, d, op, W, H)
    img_ff, ids_ff = out["far_first"]
    img_nf, ids_nf = out["near_first"]
    both = (ids_ff == 1) & (ids_nf == 0)        # the near segment wins either way
    assert both.sum() > 50
    # far first: clear -> far -> near; near first: clear -> near (the far one fails the test)
    assert not np.allclose(img_ff[both], img_nf[both], atol=1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 0])   # api.IMAGE_BLEND (the reference pipeline), api.IMAGE_NEAREST
@pytest.mark.parametrize("n,lines,segs,w,h", [(10, 12, 42, 1080, 720), (16, 5, 17, 333, 211), (32, 8, 64, 640, 480)])
def test_gpu_render_hair_matches_oracle(gpu_ctx, oracle, n, lines, segs, w, h, mode):
    """The rasterised image: the nearest segment of every pixel bit for bit,
    colours within COLOR_TOL of the oracle's; with blending, the fragments that
    pass the depth test in primitive order are decided bit for bit too."""
    import torch
    a, ns = _head(gpu_ctx, seed=n + 40, n=n)
    td = api.tess_desc_reference(n_lines=lines, n_segments=segs)
    sd = api.shade_desc_reference(image_mode=mode)
    verts, frames, depth, opac, col, (vert_d, _) = _shade_on_gpu(gpu_ctx, a, ns, n, td, sd)
    fr_d = _dev(frames.reshape(-1))
    dep_d, opa_d = _dev(depth.reshape(-1)), _dev(opac.reshape(-1))
    img = torch.full((w * h * 4,), -7.0, dtype=torch.float32, device="cuda")
    ids = torch.zeros((w * h,), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    a.render_hair(vert_d.data_ptr(), fr_d.data_ptr(), dep_d.data_ptr(), opa_d.data_ptr(), w, h, img.data_ptr(),
                  ids.data_ptr(), tess_desc=td, shade_desc=sd)
    gpu_ctx.synchronize()
    got = img.cpu().numpy().reshape(h, w, 4)
    got_ids = ids.cpu().numpy().view(np.uint32).reshape(h, w)
    want, want_ids = oracle.render_hair(verts, frames, n, lines, segs, sd, depth, opac, w, h)
    assert np.array_equal(got_ids, want_ids)
    assert (got_ids != 0xffffffff).sum() > 1000
    _colors_close(got.reshape(-1, 4), want.reshape(-1, 4))
    a.close()


def _look_at(eye, ctr, up):
    """glm::lookAt (right-handed), column-major float32."""
    eye, ctr, up = (np.asarray(x, np.float64) for x in (eye, ctr, up))
    f = (ctr - eye) / np.linalg.norm(ctr - eye)
    s_ = np.cross(f, up)
    s_ /= np.linalg.norm(s_)
    u = np.cross(s_, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s_, u, -f
    m[:3, 3] = [-s_ @ eye, -u @ eye, f @ eye]
    return m.T.astype(np.float32).reshape(-1)   # column-major


def _desc_with_camera(eye, ctr):
    sd = api.shade_desc_reference()
    for k, v in enumerate(_look_at(eye, ctr, (0.0, 1.0, 0.0))):
        sd.camera_view[k] = float(v)
    return sd


def test_oracle_raster_quad_area(oracle):
    """One straight segment seen from the front covers about its screen area in
    pixel centres: length x width, both from the projection."""
    from oracle.oracle_ctypes import render_hair
    n, L, S = 2, 1, 1
    verts = np.array([[[[-0.5, 1.0, 0.0, 0.02], [0.5, 1.0, 0.0, 0.02]]]], np.float32)   # (1, L, S+1, 4)
    frames = np.zeros((1, n - 1, 3, 4), np.float32)
    frames[0, 0, 0, :3] = (1, 0, 0)
    frames[0, 0, 1, :3] = (0, 1, 0)
    frames[0, 0, 2, :3] = (0, 0, 1)
    sd = api.shade_desc_reference(map_width=64, map_height=64)
    d, op = oracle.shade_maps(verts, sd)
    W, H = 1080, 720
    img, ids = render_hair(verts, frames, n, L, S, sd, d, op, W, H)
    hit = int((ids != 0xffffffff).sum())
    P = np.array(list(sd.camera_proj), np.float64).reshape(4, 4).T @ np.array(list(sd.camera_view),
                                                                             np.float64).reshape(4, 4).T
    c = [P @ np.array([x, 1.0, 0.0, 1.0]) for x in (-0.5, 0.5)]
    length_px = abs(c[1][0] / c[1][3] - c[0][0] / c[0][3]) * 0.5 * W
    rand = abs(np.float32(np.modf(np.sin(0.0) * 43758.5453123)[0])) + 0.5   # u = 0: random(0, 0) = 0
    width_clip = rand * 0.075 * np.linalg.norm(np.array([0.0, 1.0, 10.0]) - [-0.5, 1.0, 0.0]) * 0.02
    width_px = 2 * width_clip / c[0][3] * 0.5 * W
    assert abs(hit - length_px * width_px) <= 2 * length_px + 4, (hit, length_px, width_px)


def _near(sd):
    """The near distance of a depth-zero-to-one perspective projection."""
    m = np.array(list(sd.camera_proj), np.float64)
    return m[14] / m[10]


def _segment_image(oracle, a, b, sd, W=1080, H=720):
    """The oracle's nearest-fragment ids of one segment a -> b (one isoline)."""
    from oracle.oracle_ctypes import render_hair
    verts = np.array([[[list(a) + [0.02], list(b) + [0.02]]]], np.float32)
    frames = np.zeros((1, 1, 3, 4), np.float32)
    frames[0, 0, 0, 0] = frames[0, 0, 1, 1] = frames[0, 0, 2, 2] = 1.0
    d, op = oracle.shade_maps(verts, sd)
    return render_hair(verts, frames, 2, 1, 1, sd, d, op, W, H)[1]


def test_oracle_near_plane_clip_keeps_the_visible_part(oracle):
    """A segment running from in front of the eye to behind it is clipped at the
    near plane: it covers the pixels of the segment cut at the near plane (the
    same quad in clip space, up to the rounding of the cut point)."""
    sd = _desc_with_camera((0.0, 0.0, 0.0), (0.0, 0.0, -1.0))
    sd.image_mode = api.IMAGE_NEAREST
    near = _near(sd)
    a, b = np.array([0.03, -0.02, -1.0]), np.array([0.05, 0.06, 1.0])   # not through the eye
    t = (-near - a[2]) / (b[2] - a[2])   # eye-space z = -near: clip z = 0
    cut = a + t * (b - a)
    whole, part = _segment_image(oracle, a, b, sd) != 0xffffffff, _segment_image(oracle, a, cut, sd) != 0xffffffff
    assert part.sum() > 200
    assert (whole != part).sum() <= 0.02 * part.sum() + 4, ((whole != part).sum(), part.sum())
    behind = _segment_image(oracle, b, b + np.array([0.0, 0.05, 0.5]), sd)   # wholly behind: nothing
    assert (behind == 0xffffffff).all()


def _segment_verts(a, b, width):
    verts = np.array([[[list(a) + [width], list(b) + [width]]]], np.float32)   # (1, L = 1, S + 1 = 2, 4)
    frames = np.zeros((1, 1, 3, 4), np.float32)
    frames[0, 0, 0, 0] = frames[0, 0, 1, 1] = frames[0, 0, 2, 2] = 1.0
    return verts, frames


# one segment near the eye (0, 0, 0) looking down -z: a quad whose box is far over
# 65,536 pixels, and one running from in front of the eye to behind it
SEGMENTS = {"big": ((-0.05, -0.05, -0.15), (0.05, 0.05, -0.15), 1.0),
            "crossing": ((0.03, -0.02, -1.0), (0.05, 0.06, 1.0), 0.02)}


def test_oracle_draws_quads_over_65536_pixels(oracle):
    """A quad whose pixel box exceeds 65,536 pixels is drawn: a diagonal ribbon
    across most of the image."""
    from oracle.oracle_ctypes import render_hair
    sd = _desc_with_camera((0.0, 0.0, 0.0), (0.0, 0.0, -1.0))
    sd.image_mode = api.IMAGE_NEAREST
    a, b, width = SEGMENTS["big"]
    verts, frames = _segment_verts(a, b, width)
    d, op = oracle.shade_maps(verts, sd)
    ids = render_hair(verts, frames, 2, 1, 1, sd, d, op, 1080, 720)[1]
    hit = ids != 0xffffffff
    ys, xs = np.nonzero(hit)
    assert hit.sum() > 10000 and (xs.max() - xs.min() + 1) * (ys.max() - ys.min() + 1) > 65536


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 0])   # api.IMAGE_BLEND, api.IMAGE_NEAREST
@pytest.mark.parametrize("case", ["big", "crossing"])
def test_gpu_render_single_segment_matches_oracle(gpu_ctx, oracle, case, mode):
    """The listed quads (over 65,536 pixels, or clipped at the near plane): ids
    bit for bit, colours within COLOR_TOL of the oracle's."""
    import torch
    a, b, width = SEGMENTS[case]
    verts, frames = _segment_verts(a, b, width)
    sd = _desc_with_camera((0.0, 0.0, 0.0), (0.0, 0.0, -1.0))
    sd.image_mode = mode
    td = api.tess_desc_reference(n_lines=1, n_segments=1)
    asset = api.Asset(gpu_ctx, np.zeros((1, 24), np.float32), 2, uniform_rest=0.1)
    depth, opac = oracle.shade_maps(verts, sd)
    W, H = 1080, 720
    img = torch.zeros((W * H * 4,), dtype=torch.float32, device="cuda")
    ids = torch.zeros((W * H,), dtype=torch.int32, device="cuda")
    vd, fd = _dev(verts.reshape(-1)), _dev(frames.reshape(-1))
    dd, od = _dev(depth.reshape(-1)), _dev(opac.reshape(-1))
    torch.cuda.synchronize()
    asset.render_hair(vd.data_ptr(), fd.data_ptr(), dd.data_ptr(), od.data_ptr(), W, H, img.data_ptr(), ids.data_ptr(),
                      tess_desc=td, shade_desc=sd)
    gpu_ctx.synchronize()
    got_ids = ids.cpu().numpy().view(np.uint32).reshape(H, W)
    want, want_ids = oracle.render_hair(verts, frames, 2, 1, 1, sd, depth, opac, W, H)
    assert np.array_equal(got_ids, want_ids)
    assert (got_ids != 0xffffffff).sum() > 500
    _colors_close(img.cpu().numpy().reshape(-1, 4), want.reshape(-1, 4))
    asset.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ns", [9000, 6000, 40])
def test_gpu_blend_pixels_with_thousands_of_fragments(gpu_ctx, oracle, ns):
    """Thousands of short segments crossing one spot at random depths, drawn in
    an order unrelated to depth: pixels with more fragments than the GPU sorts
    in shared memory (8,192) take the warp-per-pixel path; ids bit for bit,
    colours within COLOR_TOL."""
    import torch
    rng = np.random.default_rng(ns)
    z = rng.uniform(-4.0, -1.0, ns)
    c = rng.uniform(-0.002, 0.002, (ns, 2)) * -z[:, None]   # about the same pixels at every depth
    a_ = np.stack([c[:, 0] - 0.01 * -z, c[:, 1] - 0.01 * -z, z], 1)
    b_ = np.stack([c[:, 0] + 0.01 * -z, c[:, 1] + 0.012 * -z, z], 1)
    verts = np.zeros((ns, 1, 2, 4), np.float32)
    verts[:, 0, 0, :3], verts[:, 0, 1, :3], verts[:, 0, :, 3] = a_, b_, 0.3
    frames = np.zeros((ns, 1, 3, 4), np.float32)
    frames[:, 0, 0, 0] = frames[:, 0, 1, 1] = frames[:, 0, 2, 2] = 1.0
    sd = _desc_with_camera((0.0, 0.0, 0.0), (0.0, 0.0, -1.0))
    sd.image_mode = api.IMAGE_BLEND
    td = api.tess_desc_reference(n_lines=1, n_segments=1)
    asset = api.Asset(gpu_ctx, np.zeros((ns, 24), np.float32), 2, uniform_rest=0.1)
    depth, opac = oracle.shade_maps(verts, sd)
    W, H = 320, 240
    img = torch.zeros((W * H * 4,), dtype=torch.float32, device="cuda")
    ids = torch.zeros((W * H,), dtype=torch.int32, device="cuda")
    vd, fd = _dev(verts.reshape(-1)), _dev(frames.reshape(-1))
    dd, od = _dev(depth.reshape(-1)), _dev(opac.reshape(-1))
    torch.cuda.synchronize()
    asset.render_hair(vd.data_ptr(), fd.data_ptr(), dd.data_ptr(), od.data_ptr(), W, H, img.data_ptr(), ids.data_ptr(),
                      tess_desc=td, shade_desc=sd)
    gpu_ctx.synchronize()
    got_ids = ids.cpu().numpy().view(np.uint32).reshape(H, W)
    want, want_ids = oracle.render_hair(verts, frames, 2, 1, 1, sd, depth, opac, W, H)
    assert np.array_equal(got_ids, want_ids)
    assert (got_ids != 0xffffffff).sum() > 20
    _colors_close(img.cpu().numpy().reshape(-1, 4), want.reshape(-1, 4))
    asset.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 0])   # api.IMAGE_BLEND, api.IMAGE_NEAREST
def test_gpu_render_hair_camera_inside_the_hair(gpu_ctx, oracle, mode):
    """A camera among the strands: quads with a corner behind it (w <= 0) are
    clipped at the near plane, quads over 65,536 pixels drawn from the list, on
    both sides the same way; ids bit for bit, colours within COLOR_TOL."""
    import torch
    a, ns = _head(gpu_ctx, seed=77, n=16)
    td = api.tess_desc_reference()
    sd = _desc_with_camera((0.0, 0.9, 0.6), (0.0, 0.2, -1.0))
    sd.image_mode = mode
    verts, frames, depth, opac, col, (vert_d, _) = _shade_on_gpu(gpu_ctx, a, ns, 16, td, sd)
    P = (np.array(list(sd.camera_proj), np.float64).reshape(4, 4).T @
         np.array(list(sd.camera_view), np.float64).reshape(4, 4).T)
    w = verts[..., :3].reshape(-1, 3).astype(np.float64) @ P[3, :3] + P[3, 3]
    w = w.reshape(verts.shape[:3])
    crossing = ((w[:, :, :-1] > 0) != (w[:, :, 1:] > 0)).sum()
    assert crossing > 10, crossing   # segments that run behind the eye: the clipped path is exercised
    fr_d, dep_d, opa_d = _dev(frames.reshape(-1)), _dev(depth.reshape(-1)), _dev(opac.reshape(-1))
    w, h = 640, 480
    img = torch.zeros((w * h * 4,), dtype=torch.float32, device="cuda")
    ids = torch.zeros((w * h,), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    a.render_hair(vert_d.data_ptr(), fr_d.data_ptr(), dep_d.data_ptr(), opa_d.data_ptr(), w, h, img.data_ptr(),
                  ids.data_ptr(), tess_desc=td, shade_desc=sd)
    gpu_ctx.synchronize()
    got_ids = ids.cpu().numpy().view(np.uint32).reshape(h, w)
    want, want_ids = oracle.render_hair(verts, frames, 16, td.n_lines, td.n_segments, sd, depth, opac, w, h)
    assert np.array_equal(got_ids, want_ids)
    assert (got_ids != 0xffffffff).sum() > 1000
    _colors_close(img.cpu().numpy().reshape(-1, 4), want.reshape(-1, 4))
    a.close()


@pytest.mark.gpu
def test_gpu_light_maps_with_the_light_inside_the_hair(gpu_ctx, oracle):
    """Light-view quads with a corner behind the light are clipped at its near
    plane: depth and opacity maps bit for bit with the oracle's."""
    a, ns = _head(gpu_ctx, seed=78, n=16)
    td = api.tess_desc_reference()
    sd = api.shade_desc_reference(map_width=540, map_height=360, map_mode=api.SHADE_MAPS_QUADS)
    for k, v in enumerate(_look_at((0.1, 0.8, 0.5), (0.0, 0.3, -1.0), (0.0, 1.0, 0.0))):
        sd.light_view[k] = float(v)
    verts, frames, depth, opac, col, _ = _shade_on_gpu(gpu_ctx, a, ns, 16, td, sd)
    want_depth, want_opac = oracle.shade_maps(verts, sd)
    assert _same_bits(depth, want_depth)
    assert _same_bits(opac, want_opac)
    assert (depth < 1).sum() > 1000
    a.close()


@pytest.mark.gpu
def test_gpu_shade_maps_without_colours(gpu_ctx, oracle):
    """colors = NULL: only the two light passes run; the maps are unchanged."""
    import torch
    a, ns = _head(gpu_ctx, seed=19, n=10)
    td, sd = api.tess_desc_reference(), api.shade_desc_reference()
    per = td.n_lines * (td.n_segments + 1)
    vert = torch.zeros((ns * per * 4,), dtype=torch.float32, device="cuda")
    fr = torch.zeros((ns * 9 * 12,), dtype=torch.float32, device="cuda")
    depth = torch.zeros((1080 * 720,), dtype=torch.float32, device="cuda")
    opac = torch.zeros((1080 * 720 * 4,), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    a.tessellate(vert.data_ptr(), fr.data_ptr(), desc=td)
    a.shade(vert.data_ptr(), fr.data_ptr(), depth.data_ptr(), opac.data_ptr(), None, tess_desc=td, shade_desc=sd)
    gpu_ctx.synchronize()
    v = vert.cpu().numpy().reshape(ns, td.n_lines, td.n_segments + 1, 4)
    want_d, want_o = oracle.shade_maps(v, sd)
    assert _same_bits(depth.cpu().numpy().reshape(720, 1080), want_d)
    assert _same_bits(opac.cpu().numpy().reshape(720, 1080, 4), want_o)
    a.close()


@pytest.mark.gpu
def test_gpu_shade_rejects_bad_arguments(gpu_ctx):
    """Every call below fails its argument checks before any launch; the buffer
    is large enough for what a launch with those arguments would touch."""
    import torch
    from rvh._lib import RvhError
    a, ns = _head(gpu_ctx, seed=1, n=8, ns=8)
    buf = torch.zeros((400 << 20) // 4, dtype=torch.float32, device="cuda")
    p = buf.data_ptr()
    for kw in ({"map_width": 0}, {"map_height": 20000}, {"map_mode": 2}):
        with pytest.raises(RvhError):
            a.shade(p, p, p, p, p, shade_desc=api.shade_desc_reference(**kw))
    sd = api.shade_desc_reference()
    sd.light_view[3] = float("nan")
    with pytest.raises(RvhError):
        a.shade(p, p, p, p, p, shade_desc=sd)
    with pytest.raises(RvhError):   # misaligned colour buffer
        a.shade(p, p, p, p, p + 4)
    with pytest.raises(RvhError):
        api.render_image(gpu_ctx, 10, p, p, 0, 10, p)
    with pytest.raises(RvhError):   # image too large
        a.render_hair(p, p, p, p, 20000, 10, p)
    with pytest.raises(RvhError):   # misaligned image
        a.render_hair(p, p, p, p, 10, 10, p + 4)
    torch.cuda.synchronize()
    a.close()
