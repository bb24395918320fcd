/*
 * hair_adjoint.hpp — TEST INFRASTRUCTURE ONLY.
 *
 * FP64 reverse-mode derivative of the hair step WITHOUT the hair-hair grid
 * (loops 1 and 2 of src/shaders/compute.comp:144-216: penalty collisions, PBD
 * predict, FTL, velocity damping and clamp, DFTL correction).  It is the CPU
 * reference for the GPU adjoint kernel.
 *
 * Loss: L = 1/ns * sum_s |x_tip,s(T) - target_s|^2 after n_steps steps.
 * Gradients: per-strand wind (3 per strand), per-strand rest segment length,
 * initial velocities (3 per point; the root's entry is 0 because the root
 * velocity is never read, compute.comp:144 starts at i = 1).
 * Piecewise rules: the contact set and the |v| > vmax branch are held fixed
 * (their indicator functions have zero derivative almost everywhere).
 * Checkpoints: the forward keeps (X, V) every CKPT steps and the reverse
 * recomputes each segment, the same schedule the GPU adjoint uses.
 */
#pragma once

#include <vector>

#include "hair_oracle.hpp"

namespace oracle {

using d3 = v3<double>;

struct Mat34 {  /* xyz rows of a column-major mat4: y = A x + b */
    double A[3][3];
    double b[3];
};
inline Mat34 mat34(const float* m) {
    Mat34 r;
    for (int row = 0; row < 3; ++row) {
        for (int col = 0; col < 3; ++col) r.A[row][col] = double(m[col * 4 + row]);
        r.b[row] = double(m[12 + row]);
    }
    return r;
}
inline d3 matT_vec(const Mat34& M, d3 v) {  /* A^T v */
    return {M.A[0][0] * v.x + M.A[1][0] * v.y + M.A[2][0] * v.z,
            M.A[0][1] * v.x + M.A[1][1] * v.y + M.A[2][1] * v.z,
            M.A[0][2] * v.x + M.A[1][2] * v.y + M.A[2][2] * v.z};
}
/* VJP of y = a/|a| at a: returns (ybar - y (y.ybar)) / |a|. */
inline d3 normalize_vjp(d3 a, d3 ybar) {
    const double len = length(a);
    const d3 y = a / len;
    return (ybar - y * dot(y, ybar)) / len;
}

constexpr int kAdjointCheckpoint = 10;

/* One forward step of one strand on compact arrays (X, V: 3*n each), through
 * the oracle's own strand_predict so the forward is the oracle's exactly. */
inline void fwd_strand(double* X, double* V, int n, double rest, d3 f0, const rvh_collider* cols, int ncol,
                       const rvh_sim_params& P, double dt) {
    double rec[12 * RVH_MAX_POINTS];
    for (int i = 0; i < n; ++i) {
        st(rec + 4 * i, mk(X[3 * i], X[3 * i + 1], X[3 * i + 2]), 1.0);
        st(rec + 4 * n + 4 * i, mk(V[3 * i], V[3 * i + 1], V[3 * i + 2]), 0.0);
        st(rec + 8 * n + 4 * i, mk(0.0, 0.0, 0.0), 0.0);
    }
    strand_predict<double>(rec, n, rest, f0, cols, ncol, P, dt);
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < 3; ++q) {
            X[3 * i + q] = rec[4 * i + q];
            V[3 * i + q] = rec[4 * n + 4 * i + q];
        }
}

/* Reverse of one step of one strand.  In: step inputs X, V and the adjoints
 * Xb, Vb of its outputs.  Out: Xb, Vb replaced by the adjoints of the inputs;
 * rest_bar and wind_bar accumulated. */
inline void rev_strand(const double* X, const double* V, double* Xb, double* Vb, int n, double r, d3 f0,
                       const rvh_collider* cols, int ncol, const rvh_sim_params& P, double dt,
                       double& rest_bar, d3& wind_bar) {
    const double k = P.k_penalty, damp = P.damping, s = P.dftl_damping, vmax = P.vmax;
    d3 x[RVH_MAX_POINTS] = {}, pred[RVH_MAX_POINTS], xn[RVH_MAX_POINTS], u[RVH_MAX_POINTS];
    int cnt[RVH_MAX_POINTS];
    for (int i = 0; i < n; ++i) x[i] = mk(X[3 * i], X[3 * i + 1], X[3 * i + 2]);
    xn[0] = x[0];
    /* recompute the forward intermediates (same formulas as strand_predict) */
    for (int i = 1; i < n; ++i) {
        d3 added = mk(0.0, 0.0, 0.0);
        int c_n = 0;
        for (int j = 0; j < ncol; ++j) {
            const rvh_collider& c = cols[j];
            if (c.kind == RVH_COLLIDER_SPHERE) {
                const d3 ctr = mk(double(c.transform[12]), double(c.transform[13]), double(c.transform[14]));
                if (distance(x[i], ctr) < double(c.radius)) {
                    added = added + (k * (double(c.radius) - distance(x[i], ctr))) * normalize(x[i] - ctr);
                    c_n++;
                }
            } else {
                const d3 q = mat_xyz(c.inv, x[i], 1.0);
                if (length(q) <= 1.0) {
                    const d3 surf = mat_xyz(c.transform, normalize(q), 1.0);
                    added = added + (k * distance(surf, x[i])) * normalize(normalize(mat_xyz(c.inv_trans, q, 0.0)));
                    c_n++;
                }
            }
        }
        d3 f = f0;
        if (c_n > 0) f = f + added / double(c_n);
        cnt[i] = c_n;
        const d3 v = mk(V[3 * i], V[3 * i + 1], V[3 * i + 2]);
        pred[i] = x[i] + dt * v + (dt * dt) * f;
        xn[i] = xn[i - 1] + r * normalize(pred[i] - xn[i - 1]);
        u[i] = damp * ((xn[i] - x[i]) / dt);
    }
    d3 xnb[RVH_MAX_POINTS], cb[RVH_MAX_POINTS], xb[RVH_MAX_POINTS], vb[RVH_MAX_POINTS], pb[RVH_MAX_POINTS];
    for (int i = 0; i < n; ++i) {
        xnb[i] = mk(Xb[3 * i], Xb[3 * i + 1], Xb[3 * i + 2]);
        cb[i] = xb[i] = vb[i] = pb[i] = mk(0.0, 0.0, 0.0);
    }
    /* v'_i = vhat_i - c_{i+1}/dt */
    for (int i = 1; i < n; ++i) {
        const d3 vob = mk(Vb[3 * i], Vb[3 * i + 1], Vb[3 * i + 2]);
        if (i != n - 1) cb[i + 1] = cb[i + 1] - vob / dt;
        /* vhat = clamp(u) */
        d3 ub = vob;
        const double ul = length(u[i]);
        if (ul > vmax) {
            const d3 uh = u[i] / ul;
            ub = (vmax / ul) * (vob - uh * dot(uh, vob));
        }
        /* u = damp (xn - x)/dt */
        xnb[i] = xnb[i] + (damp / dt) * ub;
        xb[i] = xb[i] - (damp / dt) * ub;
    }
    /* c_i = s (xn_i - pred_i) */
    for (int i = 1; i < n; ++i) {
        xnb[i] = xnb[i] + s * cb[i];
        pb[i] = pb[i] - s * cb[i];
    }
    /* FTL chain, tip to root: xn_i = xn_{i-1} + r normalize(pred_i - xn_{i-1}) */
    for (int i = n - 1; i >= 1; --i) {
        const d3 dvec = pred[i] - xn[i - 1];
        const d3 nh = normalize(dvec);
        rest_bar += dot(xnb[i], nh);
        const d3 db = normalize_vjp(dvec, r * xnb[i]);
        xnb[i - 1] = xnb[i - 1] + xnb[i] - db;
        pb[i] = pb[i] + db;
    }
    /* pred = x + dt v + dt^2 f,  f = f0 + mean penalty */
    for (int i = 1; i < n; ++i) {
        xb[i] = xb[i] + pb[i];
        vb[i] = vb[i] + dt * pb[i];
        const d3 fb = (dt * dt) * pb[i];
        wind_bar = wind_bar + fb;
        if (cnt[i] == 0) continue;
        const d3 g = fb / double(cnt[i]);
        for (int j = 0; j < ncol; ++j) {
            const rvh_collider& c = cols[j];
            if (c.kind == RVH_COLLIDER_SPHERE) {
                const d3 ctr = mk(double(c.transform[12]), double(c.transform[13]), double(c.transform[14]));
                const double R = double(c.radius);
                const double rho = distance(x[i], ctr);
                if (!(rho < R)) continue;
                const d3 e = (x[i] - ctr) / rho;
                const double eg = dot(e, g);
                xb[i] = xb[i] + k * ((-eg) * e + ((R - rho) / rho) * (g - eg * e));
            } else {
                const d3 q = mat_xyz(c.inv, x[i], 1.0);
                if (!(length(q) <= 1.0)) continue;
                const Mat34 Ainv = mat34(c.inv), Mx = mat34(c.transform), Bt = mat34(c.inv_trans);
                const d3 uh = normalize(q);
                const d3 surf = mat_xyz(c.transform, uh, 1.0);
                const d3 e = surf - x[i];
                const double d = length(e);
                const d3 m = mat_xyz(c.inv_trans, q, 0.0);
                const d3 nt = normalize(m);
                const double dbar = k * dot(nt, g);
                const d3 ntb = (k * d) * g;
                d3 qb = mk(0.0, 0.0, 0.0);
                if (d > 0.0) {
                    const d3 eb = (dbar / d) * e;
                    xb[i] = xb[i] - eb;
                    qb = qb + normalize_vjp(q, matT_vec(Mx, eb));
                }
                qb = qb + matT_vec(Bt, normalize_vjp(m, ntb));
                xb[i] = xb[i] + matT_vec(Ainv, qb);
            }
        }
    }
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < 3; ++q) {
            const double xv = (i == 0) ? 0.0 : (q == 0 ? xb[i].x : q == 1 ? xb[i].y : xb[i].z);
            const double vv = (i == 0) ? 0.0 : (q == 0 ? vb[i].x : q == 1 ? vb[i].y : vb[i].z);
            Xb[3 * i + q] = xv;
            Vb[3 * i + q] = vv;
        }
}

inline d3 strand_force0(const rvh_sim_params& P, const rvh_frame& F, const double* strand_wind, int s) {
    d3 f = mk(double(P.gravity[0]), double(P.gravity[1]), double(P.gravity[2]));
    f = f + mk(double(F.wind[0]), double(F.wind[1]), double(F.wind[2]));
    if (strand_wind) f = f + mk(strand_wind[3 * s], strand_wind[3 * s + 1], strand_wind[3 * s + 2]);
    return f;
}

inline void load_strand(const double* state0, int s, int n, double* X, double* V) {
    const double* rec = state0 + size_t(12) * n * s;
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < 3; ++q) {
            X[3 * i + q] = rec[4 * i + q];
            V[3 * i + q] = rec[4 * n + 4 * i + q];
        }
}

inline double strand_tip_loss(const double* X, int n, const double* target, int s) {
    const d3 tip = mk(X[3 * (n - 1)], X[3 * (n - 1) + 1], X[3 * (n - 1) + 2]);
    const d3 tg = mk(target[3 * s], target[3 * s + 1], target[3 * s + 2]);
    const d3 e = tip - tg;
    return dot(e, e);
}

inline double forward_loss(const double* state0, int ns, int n, const double* rest, const double* strand_wind,
                           const rvh_sim_params& P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                           int n_steps, const double* targets, int threads) {
    double total = 0.0;
#pragma omp parallel for schedule(static) num_threads(threads) reduction(+ : total) if (threads > 1)
    for (int s = 0; s < ns; ++s) {
        double X[3 * RVH_MAX_POINTS], V[3 * RVH_MAX_POINTS];
        load_strand(state0, s, n, X, V);
        for (int t = 0; t < n_steps; ++t)
            fwd_strand(X, V, n, rest[s], strand_force0(P, frames[t], strand_wind, s), cols + size_t(t) * ncol, ncol,
                       P, double(frames[t].dt));
        total += strand_tip_loss(X, n, targets, s);
    }
    return total / double(ns);
}

inline void adjoint_asset(const double* state0, int ns, int n, const double* rest, const double* strand_wind,
                          const rvh_sim_params& P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                          int n_steps, const double* targets, int threads, double* loss, double* d_wind,
                          double* d_rest, double* d_v0) {
    const int C = kAdjointCheckpoint;
    const int n_ckpt = (n_steps + C - 1) / C;
    double total = 0.0;
#pragma omp parallel for schedule(static) num_threads(threads) reduction(+ : total) if (threads > 1)
    for (int s = 0; s < ns; ++s) {
        std::vector<double> ck(size_t(n_ckpt) * 6 * n);   /* (X,V) at steps 0, C, 2C, ... */
        double X[3 * RVH_MAX_POINTS], V[3 * RVH_MAX_POINTS];
        load_strand(state0, s, n, X, V);
        for (int t = 0; t < n_steps; ++t) {
            if (t % C == 0) {
                std::copy(X, X + 3 * n, ck.begin() + size_t(t / C) * 6 * n);
                std::copy(V, V + 3 * n, ck.begin() + size_t(t / C) * 6 * n + 3 * n);
            }
            fwd_strand(X, V, n, rest[s], strand_force0(P, frames[t], strand_wind, s), cols + size_t(t) * ncol, ncol,
                       P, double(frames[t].dt));
        }
        total += strand_tip_loss(X, n, targets, s);
        double Xb[3 * RVH_MAX_POINTS] = {0}, Vb[3 * RVH_MAX_POINTS] = {0};
        const d3 tip = mk(X[3 * (n - 1)], X[3 * (n - 1) + 1], X[3 * (n - 1) + 2]);
        const d3 tg = mk(targets[3 * s], targets[3 * s + 1], targets[3 * s + 2]);
        const d3 gtip = (2.0 / double(ns)) * (tip - tg);
        Xb[3 * (n - 1)] = gtip.x; Xb[3 * (n - 1) + 1] = gtip.y; Xb[3 * (n - 1) + 2] = gtip.z;
        double rest_bar = 0.0;
        d3 wind_bar = mk(0.0, 0.0, 0.0);
        std::vector<double> seg(size_t(C) * 6 * n);          /* step inputs inside one segment */
        for (int k = n_ckpt - 1; k >= 0; --k) {
            const int t0 = k * C, t1 = std::min(n_steps, t0 + C);
            std::copy(ck.begin() + size_t(k) * 6 * n, ck.begin() + size_t(k) * 6 * n + 3 * n, X);
            std::copy(ck.begin() + size_t(k) * 6 * n + 3 * n, ck.begin() + size_t(k + 1) * 6 * n, V);
            for (int t = t0; t < t1; ++t) {
                std::copy(X, X + 3 * n, seg.begin() + size_t(t - t0) * 6 * n);
                std::copy(V, V + 3 * n, seg.begin() + size_t(t - t0) * 6 * n + 3 * n);
                if (t + 1 < t1)
                    fwd_strand(X, V, n, rest[s], strand_force0(P, frames[t], strand_wind, s), cols + size_t(t) * ncol,
                               ncol, P, double(frames[t].dt));
            }
            for (int t = t1 - 1; t >= t0; --t) {
                const double* Xi = seg.data() + size_t(t - t0) * 6 * n;
                const double* Vi = Xi + 3 * n;
                rev_strand(Xi, Vi, Xb, Vb, n, rest[s], strand_force0(P, frames[t], strand_wind, s),
                           cols + size_t(t) * ncol, ncol, P, double(frames[t].dt), rest_bar, wind_bar);
            }
        }
        if (d_rest) d_rest[s] = rest_bar;
        if (d_wind) { d_wind[3 * s] = wind_bar.x; d_wind[3 * s + 1] = wind_bar.y; d_wind[3 * s + 2] = wind_bar.z; }
        if (d_v0)
            for (int q = 0; q < 3 * n; ++q) d_v0[size_t(s) * 3 * n + q] = Vb[q];
    }
    *loss = total / double(ns);
}

}  // namespace oracle
