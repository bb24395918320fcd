"""Compile the REFERENCE's own root sampler as C++ (TEST INFRASTRUCTURE ONLY).

GeneratePointsOnMesh (src/Strand.cpp:11-146: generateRandomFloat,
generateRandomInt and the sampler) is read where it lies under the reference
checkout (the directory $RVH_REFERENCE_DIR names), cut out of
Strand.cpp in memory (the rest of that file needs Vulkan), and piped to g++
together with the reference's vendored tiny_obj_loader (src/tiny_obj_loader.h)
and glm (external/glm).  NUM_STRANDS becomes a variable the wrapper sets.  No
copy of the source is written; the only output is oracle/_ref/libref_roots.so,
exporting

    int ref_roots(const char* obj_path, int n, float* roots, float* normals)

(srand(8) and libc rand() inside, exactly as the reference runs them).
The reference cannot be built on a host without it; callers skip cleanly.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_roots.so")


def reference_dir():
    """The reference checkout named by $RVH_REFERENCE_DIR, or None."""
    return os.environ.get("RVH_REFERENCE_DIR") or None


def _paths():
    r = reference_dir()
    return (os.path.join(r, "src", "Strand.cpp"), os.path.join(r, "src", "tiny_obj_loader.h"),
            os.path.join(r, "external", "glm"))


def available():
    if reference_dir() is None:
        return False
    strand, tinyobj, glm = _paths()
    return os.path.isfile(strand) and os.path.isfile(tinyobj) and os.path.isdir(os.path.join(glm, "glm"))


PRELUDE = r"""
#include <cstdlib>
#include <string>
#include <vector>
#include <iostream>
#include <glm/glm.hpp>
#define TINYOBJLOADER_IMPLEMENTATION
#include "%s"
static int g_num_strands = 0;
#define NUM_STRANDS g_num_strands
"""

WRAPPER = r"""
extern "C" int ref_roots(const char* path, int n, float* roots, float* normals) {
    g_num_strands = n;
    std::vector<glm::vec3> p, q;
    const int r = GeneratePointsOnMesh(std::string(path), p, q);
    for (int i = 0; i < r; ++i)
        for (int a = 0; a < 3; ++a) {
            roots[3 * i + a] = p[i][a];
            normals[3 * i + a] = q[i][a];
        }
    return r;
}
"""


def extract(src):
    """The sampler and its two helpers: from generateRandomFloat up to Hair::Hair."""
    a = src.index("float generateRandomFloat()")
    b = src.index("Hair::Hair(")
    return src[a:b]


def build(force=False, verbose=False):
    """Returns the library path, or None when the reference is not present."""
    if not available():
        return None
    strand, tinyobj, glm = _paths()
    deps = [strand, tinyobj, __file__]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    with open(strand) as f:
        body = extract(f.read())
    unit = PRELUDE % tinyobj + body + WRAPPER
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-I", glm,
           "-x", "c++", "-", "-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, input=unit, text=True, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
