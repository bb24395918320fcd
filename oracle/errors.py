"""Position error against the FP64 oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/ and by bench.py's error report as the checker.

Error of a result x against the FP64 oracle y after the same steps: per curve
point |x - y| / L, L the strand's length (rest segment x (n - 1)).

Conditioning.  Over 120 steps the step is chaotic for part of the strands:
strands rooted near the crown start straight up (an inverted pendulum), the
penalty force is switched by an inside/outside test, and the grid's
int(scale * w * v) truncation is a discontinuity.  FP32 arithmetic, the
reference shader's own included, then cannot stay near FP64 on those strands.
`spread` measures this in FP64 alone: the largest deviation, over a few seeds,
of an FP64 run whose initial positions were moved by N(0, (rel * L)^2) per
coordinate (rel = 1e-7, FP32's relative precision) from the unmoved FP64 run.
A strand whose spread stays <= 1e-4 L amplifies an FP32-sized input error
less than 1000 times; such strands are "well conditioned".
"""
import numpy as np

from . import oracle_ctypes as O


def lengths(rest, n_points):
    return np.asarray(rest, np.float64) * (n_points - 1)


def point_errors(got, ref, n_points, L):
    """(ns, n) array of |x_got - x_ref| / L over the curve points."""
    a = np.asarray(got)[:, :n_points, :3].astype(np.float64)
    b = np.asarray(ref)[:, :n_points, :3].astype(np.float64)
    return np.linalg.norm(a - b, axis=2) / np.asarray(L, np.float64).reshape(-1, 1)


def summary(e):
    e = np.asarray(e, np.float64).reshape(-1)
    if e.size == 0:
        return {"max": 0.0, "p99": 0.0, "mean": 0.0, "within_1e-3": 1.0}
    return {"max": float(e.max()), "p99": float(np.percentile(e, 99)), "mean": float(e.mean()),
            "within_1e-3": float((e <= 1e-3).mean())}


def segment_error(state, rest, n_points):
    """Largest |segment length - rest| / L over every strand."""
    x = np.asarray(state)[:, :n_points, :3].astype(np.float64)
    seg = np.linalg.norm(np.diff(x, axis=1), axis=2)
    r = np.asarray(rest, np.float64)[:, None]
    return float((np.abs(seg - r) / (r * (n_points - 1))).max()) if seg.size else 0.0


def run_spec(spec, steps, dtype, threads, state=None):
    """The oracle (float64) or its FP32 twin (float32) over `steps` frames of spec."""
    st = (spec.records if state is None else state).astype(dtype).copy()
    O.run(st, spec.n_points, spec.rest, spec.params, [spec.frame(k) for k in range(steps)],
          [spec.colliders_at(k) for k in range(steps)], steps, strand_wind=spec.strand_wind, threads=threads)
    return st


def spread(spec, steps, ref64, threads, seeds=(1, 2), rel=1e-7):
    """Per-strand FP64 amplification of an FP32-sized perturbation of the
    initial positions (module docstring), relative to strand length."""
    n = spec.n_points
    L = lengths(spec.rest, n)
    out = np.zeros(spec.n_strands)
    for seed in seeds:
        p = spec.records.astype(np.float64).copy()
        rng = np.random.default_rng(seed)
        p[:, 1:n, :3] += rng.normal(0.0, rel, size=p[:, 1:n, :3].shape) * L[:, None, None]
        p = run_spec(spec, steps, np.float64, threads, state=p)
        out = np.maximum(out, point_errors(p, ref64, n, L).max(axis=1))
    return out
