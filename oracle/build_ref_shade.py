"""Compile the REFERENCE's own hair fragment shaders as C++ (TEST INFRASTRUCTURE ONLY).

Reads src/shaders/hair.frag and src/shaders/hairOpacity.frag where they lie
(under the reference checkout,
the directory $RVH_REFERENCE_DIR names), rewrites only the GLSL-only
declarations into C++ in memory and pipes the result to g++ against the
reference's vendored glm (external/glm), with the float literal and swizzle
rewrites of oracle/build_ref.py plus:
  * `uniform sampler2D name;` becomes a static Sampler2D: a float image with
    clamp-to-edge bilinear filtering (the reference's samplers are
    VK_FILTER_LINEAR + CLAMP_TO_EDGE, src/Renderer.cpp:14,1899-1902); texel
    centres at (i + 0.5) / size, full-precision float weights;
  * `layout(location = k) in/out T name;` become statics;
  * integer exponents of pow() become float literals (GLSL converts them);
  * a swizzle assigned to (`projCoords.xy = ...`) is written component by
    component (glm's swizzle proxies are rvalues once wrapped);
  * main() becomes frag_main();
  * each shader sits in a namespace of its own.
No rewritten copy is written anywhere; the only output is
oracle/_ref/libref_shade.so, exporting

    int ref_shade(int n, const float* in /* n x 24 */, const float* depth, const float* opacity,
                  int w, int h, float* out_rgba /* n x 4 */)

with per fragment: in_uv (2), in_u, in_v, in_w (3 each), in_viewDir (3),
in_lightDir (3), in_fragPosLightSpace (4), 3 unused; depth = w*h floats,
opacity = w*h float4 (layers r, g, b); and

    int ref_opacity(int n, const float* in, const float* depth, int w, int h, float* out_rgba)

(hairOpacity.frag's per-fragment output: layer values and z0), and

    int ref_cameras(float* out /* 4 x 16 */)

the camera view, camera projection, light view and light projection that
src/Camera.cpp:9-15,23-32 builds with glm for the arguments of
src/main.cpp:162-163,188-189 (column-major).
The reference cannot be built on a host without it; callers skip cleanly.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from oracle import build_ref  # noqa: E402

OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_shade.so")


def reference_dir():
    return build_ref.reference_dir()


def _shader(name="hair.frag"):
    return os.path.join(reference_dir(), "src", "shaders", name)


def available():
    return reference_dir() is not None and os.path.isfile(_shader()) and os.path.isfile(_shader("hairOpacity.frag")) and os.path.isdir(os.path.join(reference_dir(), "external", "glm", "glm"))


PRELUDE = r"""
#define GLM_FORCE_RADIANS
#define GLM_FORCE_DEPTH_ZERO_TO_ONE
#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>
#include <algorithm>
#include <cmath>
using namespace glm;
struct Sampler2D {
    const float* data = nullptr;
    int w = 1, h = 1, ch = 1;
};
static float texel(const Sampler2D& s, int x, int y, int c) {
    x = std::min(std::max(x, 0), s.w - 1);
    y = std::min(std::max(y, 0), s.h - 1);
    return s.data[(size_t(y) * s.w + x) * s.ch + c];
}
static vec4 texture(const Sampler2D& s, vec2 uv) {
    const float x = uv.x * (float)s.w - 0.5f, y = uv.y * (float)s.h - 0.5f;
    const float x0 = std::floor(x), y0 = std::floor(y);
    const float fx = x - x0, fy = y - y0;
    const int ix = (int)x0, iy = (int)y0;
    vec4 r(0.0f);
    for (int c = 0; c < s.ch; ++c) {
        const float a = texel(s, ix, iy, c) + fx * (texel(s, ix + 1, iy, c) - texel(s, ix, iy, c));
        const float b = texel(s, ix, iy + 1, c) + fx * (texel(s, ix + 1, iy + 1, c) - texel(s, ix, iy + 1, c));
        r[c] = a + fy * (b - a);
    }
    return r;
}
"""

DRIVER = r"""
extern "C" int ref_shade(int n, const float* in, const float* depth, const float* opacity, int w, int h,
                         float* out_rgba) {
    using namespace frag;
    depthSampler.data = depth; depthSampler.w = w; depthSampler.h = h; depthSampler.ch = 1;
    opacitySampler.data = opacity; opacitySampler.w = w; opacitySampler.h = h; opacitySampler.ch = 4;
    for (int i = 0; i < n; ++i) {
        const float* q = in + size_t(i) * 24;
        in_uv = vec2(q[0], q[1]);
        in_u = vec3(q[2], q[3], q[4]);
        in_v = vec3(q[5], q[6], q[7]);
        in_w = vec3(q[8], q[9], q[10]);
        in_viewDir = vec3(q[11], q[12], q[13]);
        in_lightDir = vec3(q[14], q[15], q[16]);
        in_fragPosLightSpace = vec4(q[17], q[18], q[19], q[20]);
        frag_main();
        for (int c = 0; c < 4; ++c) out_rgba[4 * i + c] = outColor[c];
    }
    return 0;
}
extern "C" int ref_opacity(int n, const float* in, const float* depth, int w, int h, float* out_rgba) {
    using namespace opac;
    depthSampler.data = depth; depthSampler.w = w; depthSampler.h = h; depthSampler.ch = 1;
    for (int i = 0; i < n; ++i) {
        const float* q = in + size_t(i) * 24;
        in_uv = vec2(q[0], q[1]);
        in_u = vec3(q[2], q[3], q[4]);
        in_v = vec3(q[5], q[6], q[7]);
        in_w = vec3(q[8], q[9], q[10]);
        in_viewDir = vec3(q[11], q[12], q[13]);
        in_lightDir = vec3(q[14], q[15], q[16]);
        in_fragPosLightSpace = vec4(q[17], q[18], q[19], q[20]);
        frag_main();
        for (int c = 0; c < 4; ++c) out_rgba[4 * i + c] = outColor[c];
    }
    return 0;
}
static void put(const glm::mat4& m, float* out) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = m[c][r];
}
extern "C" int ref_cameras(float* out) {
    const float aspect = 1080.f / 720.f;
    const glm::vec3 eye(0.0f, 1.f, 10.f);
    glm::mat4 proj = glm::perspective(glm::radians(45.0f), aspect, 0.1f, 50.0f);
    proj[1][1] *= -1;
    put(glm::lookAt(eye, glm::vec3(0.0f, 1.0f, 0.0f), glm::vec3(0.0f, 1.0f, 0.0f)), out);
    put(proj, out + 16);
    const glm::vec3 normal = glm::normalize(glm::vec3(2.f, 0.f, 1.f) - glm::vec3(0.f, 1.f, 0.f));
    glm::mat4 lproj = glm::perspective(glm::radians(60.0f), aspect, 1.f, 10.f);
    lproj[1][1] *= -1;
    put(glm::lookAt(6.5f * normal, glm::vec3(0.0f, 1.0f, 0.0f), glm::vec3(0.0f, 1.0f, 0.0f)), out + 32);
    put(lproj, out + 48);
    return 0;
}
"""


def translate(src):
    lines = [ln for ln in src.split("\n")
             if not ln.lstrip().startswith("#version") and not ln.lstrip().startswith("#extension")]
    s = "\n".join(lines)
    s = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+sampler2D\s+(\w+)\s*;", r"static Sampler2D \1;", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*(?:in|out)\s+(\w+)\s+(\w+)\s*;", r"static \1 \2;", s)
    s = re.sub(r"\bvoid\s+main\s*\(", "void frag_main(", s)
    s = re.sub(r"\bpow\(([^;]*?),\s*(\d+)\)", r"pow(\1, \2.0)", s)
    # a swizzle on the left of `=` (projCoords.xy = ...) writes the components one by one
    s = re.sub(r"(\w+)\.xy\s*=\s*([^;=]+);",
               r"{ vec2 swizzled_ = \2; \1.x = swizzled_.x; \1.y = swizzled_.y; }", s)
    s = re.sub(r"((?:\w+)(?:\[[^\[\]]*\]|\.\w+)*)\.(xyz|xy)\b",
               lambda m: ("vec3(" if m.group(2) == "xyz" else "vec2(") + m.group(0) + ")", s)
    s = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", lambda m: m.group(0) + "f", s)
    return s


def build(force=False, verbose=False):
    """Returns the library path, or None when the reference is not present."""
    if not available():
        return None
    shaders = [("frag", _shader()), ("opac", _shader("hairOpacity.frag"))]
    deps = [p for _, p in shaders] + [__file__, build_ref.__file__]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    unit = PRELUDE
    for ns, path in shaders:
        with open(path) as f:
            unit += "namespace %s {\n%s\n}  // namespace %s\n" % (ns, translate(f.read()), ns)
    unit += DRIVER
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-I", os.path.join(reference_dir(), "external", "glm"), "-x", "c++", "-", "-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, input=unit, text=True, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
