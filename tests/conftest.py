import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
PKG = os.path.join(ROOT, "realtime-vulkan-hair_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _build_once():
    import importlib.util
    spec = importlib.util.spec_from_file_location("rvh_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


@pytest.fixture(scope="session")
def librvh():
    _build_once()
    from rvh import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_ctypes
    oracle_ctypes.lib()
    return oracle_ctypes


@pytest.fixture(scope="session")
def gpu_ctx(librvh):
    from rvh import api
    ctx = api.Context(device=0, math=api.MATH_EXACT)
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def gpu_ctx_fast(librvh):
    from rvh import api
    ctx = api.Context(device=0, math=api.MATH_FAST)
    yield ctx
    ctx.close()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def rel_pos_err(a, b, n_points, length):
    """Per-point |x_a - x_b| / L over curvePoints; returns (max, p99, mean)."""
    ea = np.asarray(a)[:, :n_points, :3].astype(np.float64)
    eb = np.asarray(b)[:, :n_points, :3].astype(np.float64)
    L = np.asarray(length, np.float64).reshape(-1, 1)
    e = np.linalg.norm(ea - eb, axis=2) / L
    return float(e.max()), float(np.percentile(e, 99)), float(e.mean())
