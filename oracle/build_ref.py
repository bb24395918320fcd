"""Compile the REFERENCE's own compute shader as C++ (TEST INFRASTRUCTURE ONLY).

Reads src/shaders/compute.comp where it lies (under the reference checkout,
the directory $RVH_REFERENCE_DIR names), rewrites only the GLSL-only
declarations into C++ in memory, and pipes the result to g++ together with
oracle/ref_harness.hpp (prelude) and oracle/ref_driver.inc (dispatch loop),
against the reference's vendored glm (external/glm).  No rewritten copy of the
shader is written anywhere; the only output is oracle/_ref/libref_shader.so.

Rewrites (each keeps the shader's meaning):
  * `#version` / `#extension` lines and the `layout(local_size_x...) in;`
    line are dropped;
  * a `layout(...) uniform|buffer Name { body } inst;` block becomes a struct
    plus a static instance, and a block without an instance name puts its
    members at file scope (GLSL makes them global); an unsized array
    `T name[];` becomes a pointer bound by the driver;
  * `.xyz` / `.xy` swizzles are wrapped in vec3(...) / vec2(...) so glm's
    swizzle proxies convert before template deduction;
  * unsuffixed floating literals get an `f` suffix (GLSL literals are float).

The reference cannot be built on a host without it; callers skip cleanly.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_shader.so")


def reference_dir():
    """The reference checkout named by $RVH_REFERENCE_DIR, or None."""
    return os.environ.get("RVH_REFERENCE_DIR") or None


def available():
    r = reference_dir()
    return r is not None and (os.path.isfile(os.path.join(r, "src", "shaders", "compute.comp"))
            and os.path.isdir(os.path.join(r, "external", "glm", "glm")))


def _block(m):
    name, body, inst = m.group(2), m.group(3), m.group(4)
    body = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2;", body)
    if inst:
        return "struct %s {%s}; static %s %s;" % (name, body, name, inst)
    return body


def translate(src):
    lines = [ln for ln in src.split("\n")
             if not ln.lstrip().startswith("#version") and not ln.lstrip().startswith("#extension")]
    s = "\n".join(lines)
    s = re.sub(r"layout\s*\(\s*local_size_x[^)]*\)\s*in\s*;", "", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*(uniform|buffer)\s+(\w+)\s*\{(.*?)\}\s*(\w*)\s*;", _block, s, flags=re.S)
    s = re.sub(r"((?:\w+)(?:\[[^\[\]]*\]|\.\w+)*)\.(xyz|xy)\b",
               lambda m: ("vec3(" if m.group(2) == "xyz" else "vec2(") + m.group(0) + ")", s)
    s = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", lambda m: m.group(0) + "f", s)
    return s


def build(force=False, verbose=False):
    """Returns the library path, or None when the reference is not present."""
    if not available():
        return None
    shader = os.path.join(reference_dir(), "src", "shaders", "compute.comp")
    deps = [shader, os.path.join(HERE, "ref_harness.hpp"), os.path.join(HERE, "ref_driver.inc"), __file__]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    with open(shader) as f:
        body = translate(f.read())
    unit = '#include "%s"\n%s\n#include "%s"\n' % (
        os.path.join(HERE, "ref_harness.hpp"), body, os.path.join(HERE, "ref_driver.inc"))
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-w",
           "-I", os.path.join(reference_dir(), "external", "glm"), "-x", "c++", "-", "-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, input=unit, text=True, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
