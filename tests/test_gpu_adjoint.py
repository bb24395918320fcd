"""GPU adjoint (C ABI rvh_adjoint) wrapped in a torch.autograd.Function —
a test-only harness — checked against the FP64 CPU adjoint and against
central finite differences (h = 1e-4, 64 random parameters) evaluated in
FP64 on the oracle.  Workload: 4,096 strands x 32 points, 60 steps, no grid,
head sphere + 2 ellipsoids; loss = mean |tip - target|^2 with targets the
initial tips displaced by N(0, 0.05^2)."""
import numpy as np
import pytest

from rvh import api, configs

pytestmark = pytest.mark.gpu

STEPS = 60


class HairTipLoss:
    """torch.autograd.Function over the GPU forward + adjoint (test harness only)."""

    @staticmethod
    def make():
        import torch

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, v0, wind, rest, asset, base_records, frames, targets):
                n = asset.n_points
                rec = base_records.copy()
                rec[:, n:2 * n, :3] = v0.detach().cpu().numpy().astype(np.float32)
                asset.write(rec)
                asset.set_strand_wind(wind.detach().cpu().numpy())
                asset.set_rest_lengths(rest.detach().cpu().numpy())
                loss, dw, dr, dv = asset.adjoint(frames, targets)
                ctx.save_for_backward(torch.from_numpy(dv).double(), torch.from_numpy(dw).double(),
                                      torch.from_numpy(dr).double())
                return torch.tensor(loss, dtype=torch.float64)

            @staticmethod
            def backward(ctx, g):
                dv, dw, dr = ctx.saved_tensors
                return g * dv, g * dw, g * dr, None, None, None, None

        return _Fn


@pytest.fixture(scope="module")
def case():
    return configs.adjoint_case(n_strands=4096, n_points=32)


@pytest.fixture(scope="module")
def gpu_grads(gpu_ctx_fast, case):
    import torch
    spec, targets = case
    n = spec.n_points
    a = api.Asset(gpu_ctx_fast, spec.records, n, rest=spec.rest, strand_wind=spec.strand_wind)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    frames = [spec.frame(k) for k in range(STEPS)]
    v0 = torch.tensor(spec.records[:, n:2 * n, :3].astype(np.float64), requires_grad=True)
    wind = torch.tensor(spec.strand_wind.astype(np.float64), requires_grad=True)
    rest = torch.tensor(spec.rest.astype(np.float64), requires_grad=True)
    fn = HairTipLoss.make()
    loss = fn.apply(v0, wind, rest, a, spec.records, frames, targets)
    loss.backward()
    out = (float(loss), wind.grad.numpy(), rest.grad.numpy(), v0.grad.numpy(), a.read())
    a.close()
    return out


def _per_strand_rel(g, c):
    g = g.reshape(g.shape[0], -1)
    c = c.reshape(c.shape[0], -1)
    return np.linalg.norm(g - c, axis=1) / np.maximum(np.linalg.norm(c, axis=1), 1e-30)


def test_gpu_adjoint_matches_fp64_without_contacts(gpu_ctx_fast, case, oracle):
    """Smooth dynamics (no colliders): FP32 GPU gradients equal the FP64 adjoint to FP32 accuracy."""
    spec, targets = case
    n = spec.n_points
    sub = slice(0, 1024)
    rec = np.ascontiguousarray(spec.records[sub])
    a = api.Asset(gpu_ctx_fast, rec, n, rest=spec.rest[sub], strand_wind=spec.strand_wind[sub])
    a.set_params(spec.params)
    a.set_colliders([])
    frames = [spec.frame(k) for k in range(STEPS)]
    loss_g, dw_g, dr_g, dv_g = a.adjoint(frames, targets[sub])
    a.close()
    loss_c, dw_c, dr_c, dv_c = oracle.adjoint(rec.astype(np.float64), n, spec.rest[sub].astype(np.float64),
                                              spec.params, frames, [], STEPS, targets[sub],
                                              strand_wind=spec.strand_wind[sub].astype(np.float64), threads=16)
    assert abs(loss_g - loss_c) <= 1e-5 * abs(loss_c), (loss_g, loss_c)
    for name, g, c in (("wind", dw_g, dw_c), ("rest", dr_g, dr_c), ("v0", dv_g, dv_c)):
        rel = np.linalg.norm(g - c) / np.linalg.norm(c)
        ps = _per_strand_rel(g, c)
        print("no contacts, %s: rel L2 %.3g, per-strand median %.3g p99 %.3g" % (name, rel, np.median(ps),
                                                                                  np.percentile(ps, 99)))
        assert rel < 1e-3 and np.median(ps) < 1e-4, (name, rel, np.median(ps))


def test_gpu_adjoint_matches_fp64_cpu_adjoint(case, gpu_grads, oracle):
    """With contacts the FP32 and FP64 trajectories can cross a contact boundary at
    different steps; the per-strand gradient then differs by O(1) for that strand.
    The bulk must agree: median per-strand error at FP32 level, 90% of strands
    within 1e-2."""
    spec, targets = case
    loss_g, dw_g, dr_g, dv_g, _ = gpu_grads
    frames = [spec.frame(k) for k in range(STEPS)]
    loss_c, dw_c, dr_c, dv_c = oracle.adjoint(spec.records.astype(np.float64), spec.n_points,
                                              spec.rest.astype(np.float64), spec.params, frames, spec.colliders,
                                              STEPS, targets, strand_wind=spec.strand_wind.astype(np.float64),
                                              threads=16)
    assert abs(loss_g - loss_c) <= 1e-4 * abs(loss_c), (loss_g, loss_c)
    for name, g, c in (("wind", dw_g, dw_c), ("rest", dr_g, dr_c), ("v0", dv_g, dv_c)):
        rel = np.linalg.norm(g - c) / np.linalg.norm(c)
        ps = _per_strand_rel(g, c)
        print("%s gradient: rel L2 %.3g; per-strand median %.3g, p90 %.3g, frac<1e-2 %.3f" % (
            name, rel, np.median(ps), np.percentile(ps, 90), np.mean(ps < 1e-2)))
        assert np.median(ps) < 1e-3 and np.mean(ps < 1e-2) > 0.9, (name, rel)


def test_gpu_adjoint_matches_central_fd_fp64(case, gpu_grads, oracle):
    spec, targets = case
    _, dw_g, dr_g, dv_g, _ = gpu_grads
    n = spec.n_points
    frames = [spec.frame(k) for k in range(STEPS)]
    st0 = spec.records.astype(np.float64)
    rest = spec.rest.astype(np.float64)
    wind = spec.strand_wind.astype(np.float64)

    ns = spec.n_strands

    def L(st=st0, r=rest, w=wind, s=0):
        # strands are independent without the grid: only strand s changes, so the
        # loss difference is (1/ns) * that strand's squared tip error difference
        return oracle.loss(st[s:s + 1], n, r[s:s + 1], spec.params, frames, spec.colliders, STEPS,
                           targets[s:s + 1], strand_wind=w[s:s + 1]) / ns

    def fd(kind, s, i, q, h):
        if kind == 0:
            wp, wm = wind.copy(), wind.copy()
            wp[s, q] += h
            wm[s, q] -= h
            return (L(w=wp, s=s) - L(w=wm, s=s)) / (2 * h)
        if kind == 1:
            rp, rm = rest.copy(), rest.copy()
            rp[s] += h
            rm[s] -= h
            return (L(r=rp, s=s) - L(r=rm, s=s)) / (2 * h)
        sp, sm = st0.copy(), st0.copy()
        sp[s, n + i, q] += h
        sm[s, n + i, q] -= h
        return (L(st=sp, s=s) - L(st=sm, s=s)) / (2 * h)

    rng = np.random.default_rng(64)
    rows = []
    for j in range(64):
        kind = j % 3
        s = int(rng.integers(0, spec.n_strands))
        i, q = int(rng.integers(1, n)), int(rng.integers(0, 3))
        ad = (dw_g[s, q], dr_g[s], dv_g[s, i, q])[kind]
        rows.append((kind, fd(kind, s, i, q, 1e-4), fd(kind, s, i, q, 1e-6), ad))
    rows = np.array(rows)
    fd4, fd6, ad = rows[:, 1], rows[:, 2], rows[:, 3]
    scale = np.abs(fd6).max()
    tol = lambda ref: 2e-2 * np.abs(ref) + 1e-4 * scale
    ok4 = np.abs(fd4 - ad) <= tol(fd4)
    # where central differences at h = 1e-4 have converged (they agree with h = 1e-6),
    # the adjoint must agree with them; elsewhere h = 1e-4 straddles a contact kink
    conv = np.abs(fd4 - fd6) <= tol(fd6)
    print("FD h=1e-4: %d/64 agree with the GPU adjoint; %d/64 converged, of which %d agree; "
          "vs h=1e-6: %d/64 agree" % (ok4.sum(), conv.sum(), (ok4 & conv).sum(),
                                     (np.abs(fd6 - ad) <= tol(fd6)).sum()))
    assert conv.sum() >= 48
    assert (ok4 & conv).sum() >= conv.sum() - 1, rows[conv & ~ok4]
    assert ok4.sum() >= 56


def test_adjoint_forward_equals_the_step_kernel(gpu_ctx, case):
    """Exact mode: the adjoint's own forward replay reproduces the step kernel's
    positions bit for bit, so its loss equals the loss of 60 rvh_step calls."""
    spec, targets = case
    n = spec.n_points
    sub = slice(0, 512)
    rec = np.ascontiguousarray(spec.records[sub])
    a = api.Asset(gpu_ctx, rec, n, rest=spec.rest[sub], strand_wind=spec.strand_wind[sub])
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    frames = [spec.frame(k) for k in range(STEPS)]
    loss_adj = a.adjoint(frames, targets[sub])[0]
    for f in frames:
        a.step(f)
    tips = a.read()[:, n - 1, :3].astype(np.float64)
    tg32 = targets[sub].astype(np.float32).astype(np.float64)   # the C ABI takes float targets
    loss_fwd = float(np.mean(np.sum((tips - tg32) ** 2, axis=1)))
    assert abs(loss_adj - loss_fwd) <= 1e-12 * abs(loss_fwd)
    a.close()


def test_adjoint_rejects_grid(gpu_ctx_fast):
    from rvh._lib import RvhError
    spec = configs.full_head(n_strands=64, n_points=8, grid_res=16)
    a = api.Asset(gpu_ctx_fast, spec.records, 8, rest=spec.rest)
    a.set_params(spec.params)
    with pytest.raises(RvhError):
        a.adjoint([spec.frame(0)], np.zeros((64, 3), np.float32))
    a.close()
