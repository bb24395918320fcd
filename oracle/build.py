"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Compiles oracle_capi.cpp (hair_oracle.hpp + hair_adjoint.hpp) with g++ and
OpenMP into oracle/_build/liboracle.so.  -ffp-contract=off keeps every
multiply and add separately rounded, so x86 and Arm hosts give the same bits.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = ["oracle_capi.cpp", "hair_oracle.hpp", "hair_adjoint.hpp", "tess_oracle.hpp", "shade_oracle.hpp",
           "scene_oracle.hpp"]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    deps = [os.path.join(HERE, s) for s in SOURCES]
    deps += [os.path.join(HERE, "..", "include", h) for h in ("rvh_types.h", "rvh_scene.h")]
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-Wall", "-Wno-unknown-pragmas", os.path.join(HERE, "oracle_capi.cpp"), "-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
