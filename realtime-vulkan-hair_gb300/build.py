"""Build the GB300 hair-step library: nvcc for sm_103a, in-tree output.

Every source in csrc/ is compiled as CUDA (`-x cu`, one -gencode, -lineinfo)
in parallel and linked into rvh/_build/librvh.so with the static CUDA
runtime.  The two kernel-instantiation files are compiled once per kernel
variant (PARTS), so no single translation unit holds every kernel.  Rebuilds
only when a source or header is newer than the library.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(HERE, "..", "include")
OUT_DIR = os.path.join(HERE, "rvh", "_build")
LIB = os.path.join(OUT_DIR, "librvh.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no implicit multiply-add contraction, so every kernel that
# inlines a device function computes the same bits; fast math asks for FMA
# explicitly (fmaf in FastMath::madd).
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-I", INCLUDE]


# source -> [(object suffix, defines)]: one translation unit per kernel variant
PARTS = {
    "rvh_batch.cu": [("_L%d_%s" % (lanes, "exact" if e else "fast"), ["-DRVH_LANES=%d" % lanes, "-DRVH_EXACT=%d" % e])
                     for lanes in (1, 4, 8, 16, 32) for e in (0, 1)],
    "rvh_plain.cu": [("_N%d_%s" % (n, "exact" if e else "fast"), ["-DRVH_NFIX=%d" % n, "-DRVH_EXACT=%d" % e])
                     for n in (0, 8, 10, 16, 24, 32) for e in (0, 1)],
}


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def units():
    """(source, object basename, extra defines) of every translation unit."""
    out = []
    for s in sources():
        b = os.path.basename(s)
        for suffix, defs in PARTS.get(b, [("", [])]):
            out.append((s, b + suffix + ".o", defs))
    return out


def _compile(src, obj, defs, verbose):
    cmd = [nvcc(), "-x", "cu"] + ARCH + FLAGS + defs + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (os.path.basename(src), r.stderr[-6000:]))
    return obj


def build(force=False, verbose=False, jobs=None):
    srcs = sources()
    deps = srcs + headers() + [__file__]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps)):
        return LIB
    obj_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    hdr_t = max(os.path.getmtime(h) for h in headers() + [__file__])
    todo = []
    objs = []
    for s, ob, defs in units():
        o = os.path.join(obj_dir, ob)
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_t):
            todo.append((s, o, defs))
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for f in [ex.submit(_compile, s, o, d, verbose) for s, o, d in todo]:
            f.result()
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-6000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
