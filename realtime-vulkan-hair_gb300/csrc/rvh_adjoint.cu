// rvh_adjoint.cu — reverse-mode derivative of the hair step without the
// hair-hair grid (loops 1-2 of compute.comp:144-216: penalty collisions, PBD
// predict, FTL, velocity damping/clamp, DFTL correction), with checkpointed
// recomputation.
//
// One warp owns one strand for the whole run (strands are independent when
// the grid is off) and lane i owns curve point i (n <= 32): every per-point
// term runs in parallel across the lanes, and only the two chains along the
// strand are sequential -- the FTL chain of the forward step (run in every
// lane, the predicted points broadcast by shuffles, as the step kernel does)
// and its reverse, the tip-to-root accumulation of the FTL adjoint.  The
// forward keeps (x, v) every C steps; the reverse walks the checkpoints
// backwards, recomputes each segment's step inputs into a per-strand tape,
// then back-propagates through those steps.  Checkpoints and tape are stored
// point-major per strand, so a warp's loads and stores are contiguous.
//
// Loss: L = 1/ns * sum_s |x_tip,s(T) - target_s|^2.  Outputs dL/d(strand
// wind), dL/d(rest segment length), dL/d(initial velocity).  The contact set
// and the |v| > vmax branch are held fixed (their derivative is zero almost
// everywhere), as in the FP64 CPU adjoint the tests compare against.
#include <algorithm>
#include <vector>

#include "rvh_internal.hpp"

namespace rvh {

constexpr int kAdjThreads = 256;   // 8 strands (warps) per CTA

struct AdjDev {
    DevAsset A;                 // asset view: params, colliders, strands (initial state), rest, wind
    const rvh_frame* frames;    // per step dt / wind
    int32_t n_steps;
    int32_t ckpt;               // checkpoint interval
    int32_t n_ckpt;
    const float4* targets;      // per strand
    float4* ck;                 // n_ckpt * ns * 2n float4 (x then v)
    float4* tape;               // ckpt * ns * 2n float4
    double* loss_parts;         // per strand |tip - target|^2
    float4* d_wind;             // per strand (xyz)
    float* d_rest;              // per strand
    float4* d_v0;               // per point (xyz)
};

__device__ __forceinline__ f3 shfl3(f3 a, int src) {
    const unsigned FULL = 0xffffffffu;
    return {__shfl_sync(FULL, a.x, src), __shfl_sync(FULL, a.y, src), __shfl_sync(FULL, a.z, src)};
}

// One forward step of the warp's strand (lane i = point i): the step kernel's
// arithmetic (strand_phase_a with one point per lane), so exact math gives
// its bits.  Lanes i >= n carry zeros; the root (lane 0) never moves.
template <class M>
__device__ __forceinline__ void fwd_warp(f3& X, f3& V, int n, float r, f3 f0, const DevAsset& A, float dt) {
    const int i = threadIdx.x & 31;
    const bool moving = i >= 1 && i < n;
    const float dt2 = M::mul(dt, dt);
    const f3 force = moving ? collide_force<M>(A, X, f0) : f0;
    // predictedPos = currentPos + dt * currentVel + dt * dt * force   (compute.comp:187)
    const f3 P = v_axpy<M>(v_axpy<M>(X, dt, V), dt2, force);
    f3 par = shfl3(X, 0), XN = X;
    for (int j = 1; j < n; ++j) {   // FTL (compute.comp:191-192), the same chain in every lane
        const f3 pj = shfl3(P, j);
        par = v_axpy<M>(par, r, v_normalize<M>(v_sub<M>(pj, par)));
        if (i == j) XN = par;
    }
    f3 v = v_scale<M>(A.damping, v_div<M>(v_sub<M>(XN, X), dt));
    if (v_len<M>(v) > A.vmax) v = v_scale<M>(A.vmax, v_normalize<M>(v));
    const f3 cor = v_scale<M>(A.dftl, v_sub<M>(XN, P));
    const f3 cn = shfl3(cor, (i + 1) & 31);   // DFTL: v_i -= corr_{i+1} / dt for i < n-1 (compute.comp:213-215)
    if (i >= 1 && i < n - 1) v = v_sub<M>(v, v_div<M>(cn, dt));
    if (moving) {
        X = XN;
        V = v;
    }
}

// plain IEEE float helpers for the reverse sweep
__device__ __forceinline__ f3 a3(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 s3(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 m3(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float d3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float l3(f3 a) { return sqrtf(d3(a, a)); }
// VJP of y = a/|a|: (ybar - y (y.ybar)) / |a|
__device__ __forceinline__ f3 nvjp(f3 a, f3 yb) {
    const float len = l3(a);
    const f3 y = m3(1.0f / len, a);
    return m3(1.0f / len, s3(yb, m3(d3(y, yb), y)));
}
// A^T v for a 3x4 / 3x3 column block (rows xyz)
__device__ __forceinline__ f3 matT(const float* m, f3 v) {
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z};
}

// Reverse of one step for the warp's strand (lane i = point i).  X, V: the
// step's inputs; Xb, Vb in: adjoints of its outputs, out: adjoints of its
// inputs.  rest_bar and wind_bar collect this lane's terms (summed over the
// warp at the end of the run).
template <class M>
__device__ __forceinline__ void rev_warp(f3 X, f3 V, f3& Xb, f3& Vb, int n, float r, f3 f0, const DevAsset& A,
                                         float dt, float& rest_bar, f3& wind_bar) {
    const int i = threadIdx.x & 31;
    const bool moving = i >= 1 && i < n;
    const float k = A.k_penalty, damp = A.damping, s = A.dftl, vmax = A.vmax;
    const float dt2 = M::mul(dt, dt);
    // recompute the step: contact count, prediction, FTL, undamped-clamp input
    int cnt = 0;
    if (moving) {
        for (int j = 0; j < A.n_colliders; ++j) {
            const DevCollider& c = A.col[j];
            if (c.kind == RVH_COLLIDER_SPHERE) {
                if (v_len<M>(v_sub<M>(X, f3{c.c[0], c.c[1], c.c[2]})) < c.radius) ++cnt;
            } else {
                if (v_len<M>(mat_p1<M>(c.inv, X)) <= 1.0f) ++cnt;
            }
        }
    }
    const f3 force = moving ? collide_force<M>(A, X, f0) : f0;
    const f3 P = v_axpy<M>(v_axpy<M>(X, dt, V), dt2, force);
    f3 par = shfl3(X, 0), XN = X;
    for (int j = 1; j < n; ++j) {
        const f3 pj = shfl3(P, j);
        par = v_axpy<M>(par, r, v_normalize<M>(v_sub<M>(pj, par)));
        if (i == j) XN = par;
    }
    const f3 U = v_scale<M>(damp, v_div<M>(v_sub<M>(XN, X), dt));
    const f3 XNm = shfl3(XN, (i + 31) & 31);   // XN_{i-1}

    // velocity outputs: DFTL (corr_{i+1} of lane i+1 gets -Vb_i / dt), clamp, damping
    const f3 z = {0.f, 0.f, 0.f};
    const f3 vb_prev = shfl3(Vb, (i + 31) & 31);   // Vb_{i-1}
    f3 cb = (i >= 2 && i < n) ? m3(-1.0f, m3(1.0f / dt, vb_prev)) : z;
    f3 xnb = Xb, xb = z, vb = z, pb = z;
    if (moving) {
        f3 ub = Vb;
        const float ul = l3(U);
        if (ul > vmax) {
            const f3 uh = m3(1.0f / ul, U);
            ub = m3(vmax / ul, s3(Vb, m3(d3(uh, Vb), uh)));
        }
        xnb = a3(xnb, m3(damp / dt, ub));
        xb = s3(xb, m3(damp / dt, ub));
        xnb = a3(xnb, m3(s, cb));
        pb = s3(pb, m3(s, cb));
    }
    // FTL adjoint, tip to root: lane j's finished xnb_j gives its pb term and
    // passes xnb_j - db_j on to lane j - 1
    const f3 dv = s3(P, XNm);
    for (int j = n - 1; j >= 1; --j) {
        f3 carry = z;
        if (i == j) {
            const f3 nh = m3(1.0f / l3(dv), dv);
            rest_bar += d3(xnb, nh);
            const f3 db = nvjp(dv, m3(r, xnb));
            carry = s3(xnb, db);
            pb = a3(pb, db);
        }
        carry = shfl3(carry, j);
        if (i == j - 1) xnb = a3(xnb, carry);
    }
    // prediction and penalty-force adjoints
    if (moving) {
        xb = a3(xb, pb);
        vb = a3(vb, m3(dt, pb));
        const f3 fb = m3(dt * dt, pb);
        wind_bar = a3(wind_bar, fb);
        if (cnt > 0) {
            const f3 g = m3(1.0f / (float)cnt, fb);
            for (int j = 0; j < A.n_colliders; ++j) {
                const DevCollider& c = A.col[j];
                if (c.kind == RVH_COLLIDER_SPHERE) {
                    const f3 e0 = s3(X, f3{c.c[0], c.c[1], c.c[2]});
                    const float rho = l3(e0);
                    if (!(v_len<M>(v_sub<M>(X, f3{c.c[0], c.c[1], c.c[2]})) < c.radius)) continue;
                    const f3 e = m3(1.0f / rho, e0);
                    const float eg = d3(e, g);
                    xb = a3(xb, m3(k, a3(m3(-eg, e), m3((c.radius - rho) / rho, s3(g, m3(eg, e))))));
                } else {
                    const f3 q = mat_p1<M>(c.inv, X);
                    if (!(v_len<M>(q) <= 1.0f)) continue;
                    const f3 uh = m3(1.0f / l3(q), q);
                    const f3 surf = mat_p1<M>(c.xf, uh);
                    const f3 e = s3(surf, X);
                    const float d = l3(e);
                    const f3 m = mat_q0<M>(c.itr, q);
                    const f3 nt = m3(1.0f / l3(m), m);
                    const float dbar = k * d3(nt, g);
                    const f3 ntb = m3(k * d, g);
                    f3 qb = z;
                    if (d > 0.f) {
                        const f3 eb = m3(dbar / d, e);
                        xb = s3(xb, eb);
                        qb = a3(qb, nvjp(q, matT(c.xf, eb)));
                    }
                    qb = a3(qb, matT(c.itr, nvjp(m, ntb)));
                    xb = a3(xb, matT(c.inv, qb));
                }
            }
        }
    }
    Xb = moving ? xb : z;
    Vb = moving ? vb : z;
}

__device__ __forceinline__ f3 strand_f0(const DevAsset& A, const rvh_frame& F, int s) {
    f3 f0 = {__fadd_rn(A.gravity[0], F.wind[0]), __fadd_rn(A.gravity[1], F.wind[1]), __fadd_rn(A.gravity[2], F.wind[2])};
    if (A.strand_wind) {
        const float4 w = A.strand_wind[s];
        f0 = {__fadd_rn(f0.x, w.x), __fadd_rn(f0.y, w.y), __fadd_rn(f0.z, w.z)};
    }
    return f0;
}

template <class M>
__global__ void __launch_bounds__(kAdjThreads) k_adjoint(const __grid_constant__ AdjDev D) {
    const DevAsset& A = D.A;
    const int s = (int)((blockIdx.x * (unsigned)kAdjThreads + threadIdx.x) >> 5);   // the warp's strand
    if (s >= A.n_strands) return;   // uniform across the warp
    const int n = A.n_points;
    const int i = threadIdx.x & 31;
    const bool live = i < n;
    const float r = A.rest[s];
    const float4* rec = A.strands + (size_t)s * 3 * n;
    f3 X = live ? xyz(rec[i]) : f3{0.f, 0.f, 0.f};
    f3 V = live ? xyz(rec[n + i]) : f3{0.f, 0.f, 0.f};
    const size_t stride = (size_t)2 * n;  // float4 per strand per saved state
    auto save = [&](float4* base, int slot) {
        if (!live) return;
        float4* p = base + ((size_t)slot * A.n_strands + s) * stride;
        p[i] = make_float4(X.x, X.y, X.z, 0.f);
        p[n + i] = make_float4(V.x, V.y, V.z, 0.f);
    };
    auto load = [&](const float4* base, int slot, f3& Xo, f3& Vo) {
        if (!live) return;
        const float4* p = base + ((size_t)slot * A.n_strands + s) * stride;
        Xo = xyz(p[i]);
        Vo = xyz(p[n + i]);
    };
    for (int t = 0; t < D.n_steps; ++t) {
        if (t % D.ckpt == 0) save(D.ck, t / D.ckpt);
        fwd_warp<M>(X, V, n, r, strand_f0(A, D.frames[t], s), A, D.frames[t].dt);
    }
    const float4 tg = D.targets[s];
    const f3 tip = shfl3(X, n - 1);
    if (i == 0) {
        const double ex = (double)tip.x - (double)tg.x, ey = (double)tip.y - (double)tg.y,
                     ez = (double)tip.z - (double)tg.z;
        D.loss_parts[s] = ex * ex + ey * ey + ez * ez;
    }
    const float g2 = 2.0f / (float)A.n_strands;
    f3 Xb = {0.f, 0.f, 0.f}, Vb = {0.f, 0.f, 0.f};
    if (i == n - 1) Xb = {g2 * (X.x - tg.x), g2 * (X.y - tg.y), g2 * (X.z - tg.z)};
    float rest_bar = 0.f;
    f3 wind_bar = {0.f, 0.f, 0.f};
    for (int k = D.n_ckpt - 1; k >= 0; --k) {
        const int t0 = k * D.ckpt, t1 = min(D.n_steps, t0 + D.ckpt);
        load(D.ck, k, X, V);
        for (int t = t0; t < t1; ++t) {
            save(D.tape, t - t0);
            if (t + 1 < t1) fwd_warp<M>(X, V, n, r, strand_f0(A, D.frames[t], s), A, D.frames[t].dt);
        }
        for (int t = t1 - 1; t >= t0; --t) {
            f3 Xi = {0.f, 0.f, 0.f}, Vi = {0.f, 0.f, 0.f};
            load(D.tape, t - t0, Xi, Vi);
            rev_warp<M>(Xi, Vi, Xb, Vb, n, r, strand_f0(A, D.frames[t], s), A, D.frames[t].dt, rest_bar, wind_bar);
        }
    }
    const unsigned FULL = 0xffffffffu;
    for (int o = 16; o > 0; o >>= 1) {   // the lanes' rest and wind terms
        rest_bar += __shfl_xor_sync(FULL, rest_bar, o);
        wind_bar.x += __shfl_xor_sync(FULL, wind_bar.x, o);
        wind_bar.y += __shfl_xor_sync(FULL, wind_bar.y, o);
        wind_bar.z += __shfl_xor_sync(FULL, wind_bar.z, o);
    }
    if (i == 0) {
        D.d_rest[s] = rest_bar;
        D.d_wind[s] = make_float4(wind_bar.x, wind_bar.y, wind_bar.z, 0.f);
    }
    if (live) D.d_v0[(size_t)s * n + i] = make_float4(Vb.x, Vb.y, Vb.z, 0.f);
}

}  // namespace rvh

using namespace rvh;

extern "C" {

rvh_status rvh_adjoint(rvh_asset* a, const rvh_frame* frames, int32_t n_steps, int32_t checkpoint_every,
                       const float* targets, double* loss, float* d_wind, float* d_rest, float* d_v0) {
    TraceRange trace("rvh_adjoint");
    if (!a || !frames || !targets || !loss) return fail(RVH_ERR_INVALID_ARG, "adjoint: NULL argument");
    if (n_steps < 1) return fail(RVH_ERR_INVALID_ARG, "adjoint: n_steps must be >= 1");
    if (checkpoint_every < 1) checkpoint_every = 10;
    if (a->params.grid_enabled)
        return fail(RVH_ERR_UNSUPPORTED, "adjoint: the hair-hair grid must be disabled (FTL+DFTL+collisions only)");
    if (a->head_active) return fail(RVH_ERR_UNSUPPORTED, "adjoint: a kinematic head motion is set");
    for (int t = 0; t < n_steps; ++t) {
        rvh_status st = validate_frame(frames[t]);
        if (st != RVH_OK) return st;
    }
    Context* ctx = a->ctx;
    RVH_DEVICE(ctx->device);
    const int ns = a->n_strands, n = a->n_points;
    if (ns == 0) {
        *loss = 0.0;
        return RVH_OK;
    }
    const int C = std::min(checkpoint_every, n_steps);
    const int n_ckpt = (n_steps + C - 1) / C;
    DevBuf fr, tg, ck, tape, lp, dw, dr, dv;
    auto cleanup = [&]() {
        for (DevBuf* b : {&fr, &tg, &ck, &tape, &lp, &dw, &dr, &dv}) ctx->free(*b);
    };
    rvh_status st;
    const size_t state = size_t(ns) * 2 * n * sizeof(float4);
    if ((st = ctx->alloc(fr, sizeof(rvh_frame) * n_steps)) || (st = ctx->alloc(tg, sizeof(float4) * ns)) ||
        (st = ctx->alloc(ck, state * n_ckpt)) || (st = ctx->alloc(tape, state * C)) ||
        (st = ctx->alloc(lp, sizeof(double) * ns)) || (st = ctx->alloc(dw, sizeof(float4) * ns)) ||
        (st = ctx->alloc(dr, sizeof(float) * ns)) || (st = ctx->alloc(dv, sizeof(float4) * size_t(ns) * n))) {
        cleanup();
        return st;
    }
    std::vector<float4> t4(ns);
    for (int s = 0; s < ns; ++s) t4[s] = make_float4(targets[3 * s], targets[3 * s + 1], targets[3 * s + 2], 0.f);
    cudaError_t e = cudaMemcpy(fr.ptr, frames, sizeof(rvh_frame) * n_steps, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(tg.ptr, t4.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(e, "adjoint upload");
    }
    AdjDev D{};
    D.A = a->device_view(frames[0], -1);
    D.frames = static_cast<const rvh_frame*>(fr.ptr);
    D.n_steps = n_steps;
    D.ckpt = C;
    D.n_ckpt = n_ckpt;
    D.targets = static_cast<const float4*>(tg.ptr);
    D.ck = static_cast<float4*>(ck.ptr);
    D.tape = static_cast<float4*>(tape.ptr);
    D.loss_parts = static_cast<double*>(lp.ptr);
    D.d_wind = static_cast<float4*>(dw.ptr);
    D.d_rest = static_cast<float*>(dr.ptr);
    D.d_v0 = static_cast<float4*>(dv.ptr);
    void* args[] = {&D};
    const void* kern = ctx->math == RVH_MATH_EXACT ? reinterpret_cast<const void*>(&k_adjoint<ExactMath>)
                                                   : reinterpret_cast<const void*>(&k_adjoint<FastMath>);
    const int per_cta = kAdjThreads / 32;   // one warp per strand
    e = cudaLaunchKernel(kern, dim3(unsigned((ns + per_cta - 1) / per_cta)), dim3(kAdjThreads), args, 0, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    std::vector<double> parts(ns);
    std::vector<float4> w4(ns), v4(size_t(ns) * n);
    std::vector<float> r1(ns);
    if (e == cudaSuccess) e = cudaMemcpy(parts.data(), lp.ptr, sizeof(double) * ns, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(w4.data(), dw.ptr, sizeof(float4) * ns, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(r1.data(), dr.ptr, sizeof(float) * ns, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(v4.data(), dv.ptr, sizeof(float4) * v4.size(), cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(e, "adjoint");
    double sum = 0.0;
    for (double p : parts) sum += p;
    *loss = sum / double(ns);
    if (d_wind)
        for (int s = 0; s < ns; ++s) {
            d_wind[3 * s] = w4[s].x;
            d_wind[3 * s + 1] = w4[s].y;
            d_wind[3 * s + 2] = w4[s].z;
        }
    if (d_rest) std::copy(r1.begin(), r1.end(), d_rest);
    if (d_v0)
        for (size_t p = 0; p < v4.size(); ++p) {
            d_v0[3 * p] = v4[p].x;
            d_v0[3 * p + 1] = v4[p].y;
            d_v0[3 * p + 2] = v4[p].z;
        }
    return RVH_OK;
}

}  // extern "C"
