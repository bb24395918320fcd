"""The oracle's FP64 adjoint (no grid: FTL + DFTL + collisions) agrees with
central finite differences of the FP64 oracle loss.  CPU only.

h = 1e-7: the FP64 loss is accurate to ~1e-16, so the FD rounding error is
~1e-9 and the truncation error O(h^2) stays small even for strands whose
loss is strongly nonlinear."""
import numpy as np
import pytest

from rvh import configs


def _case(ns=48, n=16, steps=30, seed=4):
    spec, targets = configs.adjoint_case(n_strands=ns, n_points=n, seed=seed)
    frames = [spec.frame(k) for k in range(steps)]
    return spec, targets, frames, steps


@pytest.mark.parametrize("steps", [1, 25])
def test_fp64_adjoint_matches_central_fd(oracle, steps):
    spec, targets, frames, _ = _case(steps=steps)
    n = spec.n_points
    st0 = spec.records.astype(np.float64)
    rest = spec.rest.astype(np.float64)
    wind = spec.strand_wind.astype(np.float64)
    loss, dw, dr, dv = oracle.adjoint(st0, n, rest, spec.params, frames, spec.colliders, steps, targets,
                                      strand_wind=wind, threads=4)
    L0 = oracle.loss(st0, n, rest, spec.params, frames, spec.colliders, steps, targets, strand_wind=wind)
    assert abs(loss - L0) <= 1e-12 * max(1.0, abs(L0))
    rng = np.random.default_rng(0)
    h = 1e-7
    checks = []
    for _ in range(24):
        kind = rng.integers(0, 3)
        s = int(rng.integers(0, spec.n_strands))
        if kind == 0:
            q = int(rng.integers(0, 3))
            wp, wm = wind.copy(), wind.copy()
            wp[s, q] += h
            wm[s, q] -= h
            fd = (oracle.loss(st0, n, rest, spec.params, frames, spec.colliders, steps, targets, strand_wind=wp)
                  - oracle.loss(st0, n, rest, spec.params, frames, spec.colliders, steps, targets, strand_wind=wm)) / (2 * h)
            ad = dw[s, q]
        elif kind == 1:
            rp, rm = rest.copy(), rest.copy()
            rp[s] += h
            rm[s] -= h
            fd = (oracle.loss(st0, n, rp, spec.params, frames, spec.colliders, steps, targets, strand_wind=wind)
                  - oracle.loss(st0, n, rm, spec.params, frames, spec.colliders, steps, targets, strand_wind=wind)) / (2 * h)
            ad = dr[s]
        else:
            i = int(rng.integers(1, n))
            q = int(rng.integers(0, 3))
            sp, sm = st0.copy(), st0.copy()
            sp[s, n + i, q] += h
            sm[s, n + i, q] -= h
            fd = (oracle.loss(sp, n, rest, spec.params, frames, spec.colliders, steps, targets, strand_wind=wind)
                  - oracle.loss(sm, n, rest, spec.params, frames, spec.colliders, steps, targets, strand_wind=wind)) / (2 * h)
            ad = dv[s, i, q]
        checks.append((kind, fd, ad))
    scale = max(abs(c[1]) for c in checks)
    bad = [c for c in checks if abs(c[1] - c[2]) > 1e-5 * scale + 1e-6 * abs(c[1])]
    assert len(bad) <= 1, bad   # one kink crossing (contact set change) is tolerated
    assert np.all(dv[:, 0] == 0.0)
