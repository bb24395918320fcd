"""Compile the REFERENCE's own tessellation shader as C++ (TEST INFRASTRUCTURE ONLY).

Reads src/shaders/hair.tese where it lies (under the reference checkout,
the directory $RVH_REFERENCE_DIR names), rewrites only the GLSL-only
declarations into C++ in memory and pipes the result to g++ against the
reference's vendored glm (external/glm), with the float literal, swizzle and
uniform-block rewrites of oracle/build_ref.py plus:
  * `layout(isolines) in;` is dropped;
  * the patch input `vec4[][NUM_CURVE_POINTS] in_curvePoints` becomes a static
    array of 3 patch vertices x (NUM_CURVE_POINTS + 2) points, zero-padded so
    the shader's out-of-bounds read at v = 1 reads zeros;
  * `layout(location = k) out T name;` outputs become statics, `out T name`
    parameters references, and gl_TessCoord / gl_Position statics;
  * main() becomes tese_main().
No rewritten copy is written anywhere; the only output is
oracle/_ref/libref_tess.so, exporting

    int ref_tess(const float* records, int ns, int n_lines, int n_segments,
                 float* out, float* frames)

for strands of NUM_CURVE_POINTS (10) points: out = ns * n_lines *
(n_segments + 1) float4 {gl_Position.xyz, out_strandWidth}; frames = ns *
n_lines * (n_segments + 1) * 9 floats {out_u, out_v, out_w}.
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
LIB = os.path.join(OUT_DIR, "libref_tess.so")


def reference_dir():
    return build_ref.reference_dir()


def _shader():
    return os.path.join(reference_dir(), "src", "shaders", "hair.tese")


def available():
    return reference_dir() is not None and os.path.isfile(_shader()) and os.path.isdir(os.path.join(reference_dir(), "external", "glm", "glm"))


PRELUDE = r"""
#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>
#include <glm/gtc/matrix_inverse.hpp>
using namespace glm;
static vec3 gl_TessCoord;
static vec4 gl_Position;
"""

DRIVER = r"""
extern "C" int ref_tess(const float* records, int ns, int n_lines, int n_segments, float* out, float* frames) {
    const int n = NUM_CURVE_POINTS;
    camera.view = mat4(1.0f); camera.proj = mat4(1.0f);
    shadowCamera.view = mat4(1.0f); shadowCamera.proj = mat4(1.0f);
    for (int s = 0; s < ns; ++s) {
        for (int p = 0; p < 3; ++p)
            for (int i = 0; i < n + 2; ++i) in_curvePoints[p][i] = vec4(0.0f);
        for (int i = 0; i < n; ++i) {
            const float* q = records + (size_t(s) * 12 * n + 4 * i);
            in_curvePoints[0][i] = vec4(q[0], q[1], q[2], q[3]);
        }
        for (int j = 0; j < n_lines; ++j)
            for (int k = 0; k <= n_segments; ++k) {
                gl_TessCoord = vec3((float)k / (float)n_segments, (float)j / (float)n_lines, 0.0f);
                tese_main();
                const size_t o = (size_t(s) * n_lines + j) * (n_segments + 1) + k;
                out[4 * o] = gl_Position.x; out[4 * o + 1] = gl_Position.y; out[4 * o + 2] = gl_Position.z;
                out[4 * o + 3] = out_strandWidth;
                if (frames) {
                    const vec3 f[3] = {out_u, out_v, out_w};
                    for (int q = 0; q < 3; ++q)
                        for (int a = 0; a < 3; ++a) frames[9 * o + 3 * q + a] = f[q][a];
                }
            }
    }
    return 0;
}
"""


def translate(src):
    lines = [ln for ln in src.split("\n")
             if not ln.lstrip().startswith("#version") and not ln.lstrip().startswith("#extension")]
    s = "\n".join(lines)
    s = re.sub(r"layout\s*\(\s*isolines\s*\)\s*in\s*;", "", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*(uniform|buffer)\s+(\w+)\s*\{(.*?)\}\s*(\w*)\s*;", build_ref._block, s, flags=re.S)
    s = re.sub(r"layout\s*\([^)]*\)\s*in\s+vec4\s*\[\s*\]\s*\[\s*NUM_CURVE_POINTS\s*\]\s*(\w+)\s*;",
               r"static vec4 \1[3][NUM_CURVE_POINTS + 2];", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*out\s+(\w+)\s+(\w+)\s*;", r"static \1 \2;", s)
    s = re.sub(r"\bout\s+(\w+)\s+(\w+)\s*([,)])", r"\1& \2\3", s)
    s = re.sub(r"\bvoid\s+main\s*\(", "void tese_main(", s)
    s = re.sub(r"((?:\w+)(?:\[[^\[\]]*\]|\.\w+)*)\.(xyz|xy)\b",
               lambda m: ("vec3(" if m.group(2) == "xyz" else "vec2(") + m.group(0) + ")", s)
    s = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", lambda m: m.group(0) + "f", s)
    return s


def build(force=False, verbose=False):
    """Returns the library path, or None when the reference is not present."""
    if not available():
        return None
    shader = _shader()
    deps = [shader, __file__, build_ref.__file__]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    with open(shader) as f:
        unit = PRELUDE + translate(f.read()) + DRIVER
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
