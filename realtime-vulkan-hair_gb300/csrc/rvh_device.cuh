// rvh_device.cuh — device-side data layout and the per-strand / per-point step
// functions of the GB300 hair step.  Every kernel (plain per-asset launches,
// the batched persistent launch) calls these, so they compute identical bits.
//
// Reference: clach/Realtime-Vulkan-Hair src/shaders/compute.comp:124-303.
//   loop 1 (:144-202)  predict + penalty collisions + FTL     -> phase A
//   loop 2 (:211-253)  DFTL velocity correction + grid splat  -> phase A
//   loop 3 (:257-298)  grid gather + friction (+ repulsion)   -> phase B
// Phase B of an asset starts only after every phase-A tile of that asset has
// splatted (a global phase split; the shader's barrier() is workgroup-only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rvh_types.h"

namespace rvh {

// ---------------------------------------------------------------------------
// Arithmetic policies.
//   Exact: every + - * / sqrt is a separately rounded IEEE operation in the
//          order the oracle writes it (no FMA contraction), so a step is
//          bit-identical to the oracle's FP32 twin.
//   Fast:  FMA contraction and approximate reciprocal / rsqrt; results stay
//          within the FP64 tolerances, at fewer instructions.
// ---------------------------------------------------------------------------
struct ExactMath {
    static constexpr bool kExact = true;
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
    static __device__ __forceinline__ float rsqrt(float a) { return __fdiv_rn(1.0f, __fsqrt_rn(a)); }
    static __device__ __forceinline__ float rcp(float a) { return __fdiv_rn(1.0f, a); }
    // a*b + c written as two roundings, as the oracle does
    static __device__ __forceinline__ float madd(float a, float b, float c) { return __fadd_rn(__fmul_rn(a, b), c); }
};

struct FastMath {
    static constexpr bool kExact = false;
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return sqrtf(a); }
    static __device__ __forceinline__ float rsqrt(float a) { return rsqrtf(a); }
    static __device__ __forceinline__ float rcp(float a) { return __frcp_rn(a); }
    static __device__ __forceinline__ float madd(float a, float b, float c) { return fmaf(a, b, c); }
};

// ---------------------------------------------------------------------------
// Device layout.
// ---------------------------------------------------------------------------

// One collider, repacked from rvh_collider (three column-major mat4,
// src/Scene.h:23-27) into the 3x4 / 3x3 blocks the shader reads.
struct DevCollider {
    int32_t kind;
    float radius;    // sphere: its radius; ellipsoid: a bounding-sphere radius (largest column of
                     // the transform's 3x3, enlarged by 1e-3) used only to skip far points
    float c[3];      // centre: transform[3].xyz (compute.comp:162)
    float inv[12];   // inv, columns 0..3, rows xyz: local = inv * (p, 1) (compute.comp:65)
    float itr[9];    // invTrans, columns 0..2, rows xyz: n = invTrans * (q, 0) (compute.comp:72)
    float xf[12];    // transform, columns 0..3, rows xyz (compute.comp:78)
};

// Everything one step of one asset reads besides its buffers' contents.
struct DevAsset {
    float4* strands;             // n_strands records of 3*n float4 (Strand.h:11-15), updated in place
    const float* rest;           // per-strand rest segment length (compute.comp:139-140)
    const float4* strand_wind;   // optional per-strand wind (xyz), or null
    unsigned long long* grid;    // 4 x int64 per cell {vx, vy, vz, density}: this step's splat target, or the
                                 // grid a phase-B (gather-only) tile reads
    unsigned long long* grid_next;  // the buffer a batched step clears for a later step
    unsigned long long* grid_prev;  // fused batched step: the previous step's splat, whose gather + friction
                                    // this pass applies before stepping (null: nothing pending)
    rvh_draw_indirect* draw;     // StrandDrawIndirect (Strand.h:53-58), or null
    int32_t n_strands;
    int32_t n_points;
    // constants (rvh_sim_params)
    float gravity[3];
    float damping, dftl, vmax, k_penalty, friction, repulsion, scale;
    int32_t grid_enabled, wrap32;
    float origin[3];
    float h;
    float inv_h;                 // 1 / h (fast math maps positions to grid space by a multiply)
    int32_t nx, ny, nz;
    // frame (rvh_frame)
    float dt_prev;               // dt of the step whose friction is pending (with grid_prev)
    float dt;
    float t;
    float wind[3];
    int32_t n_colliders;
    DevCollider col[RVH_MAX_COLLIDERS];
    // kinematic head: with root_rest set, each strand's root is placed at head * root_rest
    // (head: row-major 3 x 4 affine) before the FTL chain
    const float4* root_rest;
    float head[12];
    // optional: the step also writes every point's new position (xyz, the root
    // included) to pos_xyz[3 * (strand * n + i)], for a device-to-host copy
    float* pos_xyz;
    // Cell boxes of the phase-A groups (two int4 per group, indexed by the
    // group's first round: {lo xyz, tag}, {hi xyz, points}).  A fused step
    // writes each group's splat box under box_tag_write; the next fused step
    // of the same grouping finds there the box of the positions its pending
    // gather reads (the same points, unmoved since) when the tag equals
    // box_tag_read, and skips recomputing it.  Null or tag 0: not used.
    int4* group_box;
    uint32_t box_tag_read;
    uint32_t box_tag_write;
    // rounds per phase-A group (the span of one gather box and one splat box);
    // 0: as many as keep a group's density partials exact, at most 4
    int32_t group_rounds;
    // a later step of the same asset in one launch: its phase-A and clear items
    // start only once every phase-A and clear item of entry wait_entry (the
    // asset's previous step) is done; -1: none
    int32_t wait_entry;
};

struct f3 {
    float x, y, z;
};

template <class M> __device__ __forceinline__ f3 v_add(f3 a, f3 b) { return {M::add(a.x, b.x), M::add(a.y, b.y), M::add(a.z, b.z)}; }
template <class M> __device__ __forceinline__ f3 v_sub(f3 a, f3 b) { return {M::sub(a.x, b.x), M::sub(a.y, b.y), M::sub(a.z, b.z)}; }
template <class M> __device__ __forceinline__ f3 v_scale(float s, f3 a) { return {M::mul(s, a.x), M::mul(s, a.y), M::mul(s, a.z)}; }
template <class M> __device__ __forceinline__ f3 v_div(f3 a, float s) { return {M::div(a.x, s), M::div(a.y, s), M::div(a.z, s)}; }
// a + s*b
template <class M> __device__ __forceinline__ f3 v_axpy(f3 a, float s, f3 b) {
    return {M::madd(s, b.x, a.x), M::madd(s, b.y, a.y), M::madd(s, b.z, a.z)};
}
template <class M> __device__ __forceinline__ float v_dot(f3 a, f3 b) {
    return M::madd(a.z, b.z, M::madd(a.y, b.y, M::mul(a.x, b.x)));   // (ax bx + ay by) + az bz
}
template <class M> __device__ __forceinline__ float v_len(f3 a) { return M::sqrt(v_dot<M>(a, a)); }
// GLSL normalize: x * inversesqrt(dot(x, x))
template <class M> __device__ __forceinline__ f3 v_normalize(f3 a) { return v_scale<M>(M::rsqrt(v_dot<M>(a, a)), a); }

// Fast math on Blackwell's paired FP32 instructions: x and y of a vector in one
// f32x2 operation, z alone.  Each half is rounded as its scalar operation
// would be, so the results are the bits of the scalar code, in fewer
// instructions (about 8 % fewer FP32 instructions in the step kernels).
__device__ __forceinline__ unsigned long long pk2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(unsigned long long r, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
template <> __device__ __forceinline__ f3 v_add<FastMath>(f3 a, f3 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk2(a.x, a.y)), "l"(pk2(b.x, b.y)));
    f3 o;
    upk2(r, o.x, o.y);
    o.z = a.z + b.z;
    return o;
}
template <> __device__ __forceinline__ f3 v_sub<FastMath>(f3 a, f3 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk2(a.x, a.y)), "l"(pk2(b.x, b.y)));
    f3 o;
    upk2(r, o.x, o.y);
    o.z = a.z - b.z;
    return o;
}
template <> __device__ __forceinline__ f3 v_scale<FastMath>(float s, f3 a) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk2(s, s)), "l"(pk2(a.x, a.y)));
    f3 o;
    upk2(r, o.x, o.y);
    o.z = s * a.z;
    return o;
}
template <> __device__ __forceinline__ f3 v_axpy<FastMath>(f3 a, float s, f3 b) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pk2(s, s)), "l"(pk2(b.x, b.y)), "l"(pk2(a.x, a.y)));
    f3 o;
    upk2(r, o.x, o.y);
    o.z = fmaf(s, b.z, a.z);
    return o;
}

// xyz of m * (p, 1) for a 3x4 column block: (c0 x + c1 y) + (c2 z + c3)
template <class M> __device__ __forceinline__ f3 mat_p1(const float* m, f3 p) {
    return {M::add(M::madd(m[3], p.y, M::mul(m[0], p.x)), M::madd(m[6], p.z, m[9])),
            M::add(M::madd(m[4], p.y, M::mul(m[1], p.x)), M::madd(m[7], p.z, m[10])),
            M::add(M::madd(m[5], p.y, M::mul(m[2], p.x)), M::madd(m[8], p.z, m[11]))};
}
// xyz of m * (q, 0) for a 3x3 column block: (c0 x + c1 y) + c2 z
template <class M> __device__ __forceinline__ f3 mat_q0(const float* m, f3 q) {
    return {M::madd(m[6], q.z, M::madd(m[3], q.y, M::mul(m[0], q.x))),
            M::madd(m[7], q.z, M::madd(m[4], q.y, M::mul(m[1], q.x))),
            M::madd(m[8], q.z, M::madd(m[5], q.y, M::mul(m[2], q.x)))};
}

__device__ __forceinline__ f3 xyz(float4 a) { return {a.x, a.y, a.z}; }

// Streaming 16-B load that skips L1: data written by other CTAs in the same
// launch (phase A output, grid sums) must not be served from a stale L1 line.
__device__ __forceinline__ float4 ld_cg(const float4* p) { return __ldcg(p); }
__device__ __forceinline__ void st_f4(float4* p, f3 a, float w) { *p = make_float4(a.x, a.y, a.z, w); }

// ---------------------------------------------------------------------------
// Penalty collisions for one point (compute.comp:155-184).  Returns the force.
// ---------------------------------------------------------------------------
template <class M>
__device__ __forceinline__ f3 collide_force(const DevAsset& A, f3 x, f3 force) {
    const float k = A.k_penalty;
    f3 added = {0.f, 0.f, 0.f};
    int cnt = 0;
    const int nc = A.n_colliders;
    for (int j = 0; j < nc; ++j) {
        const DevCollider& c = A.col[j];
        if (c.kind == RVH_COLLIDER_SPHERE) {
            const f3 e = v_sub<M>(x, f3{c.c[0], c.c[1], c.c[2]});
            const float d2 = v_dot<M>(e, e);
            // clearly outside: sqrt(d2) >= r whenever d2 > r^2 (1 + 1e-5); skips the sqrt
            if (d2 > c.radius * c.radius * 1.00001f) continue;
            const float dist = M::sqrt(d2);
            if (dist < c.radius) {
                const float d = M::sub(c.radius, dist);
                const f3 nrm = v_normalize<M>(e);
                added = v_axpy<M>(added, M::mul(k, d), nrm);
                ++cnt;
            }
        } else {
            // outside the bounding sphere: the exact test below would fail too
            const f3 e = v_sub<M>(x, f3{c.c[0], c.c[1], c.c[2]});
            if (v_dot<M>(e, e) > c.radius * c.radius) continue;
            const f3 q = mat_p1<M>(c.inv, x);
            const float q2 = v_dot<M>(q, q);
            if (q2 > 1.00001f) continue;   // clearly outside (sqrt(q2) > 1)
            const float lq = M::sqrt(q2);
            if (lq <= 1.0f) {
                const f3 surf = mat_p1<M>(c.xf, v_normalize<M>(q));
                const float d = v_len<M>(v_sub<M>(surf, x));
                const f3 nrm = v_normalize<M>(v_normalize<M>(mat_q0<M>(c.itr, q)));
                added = v_axpy<M>(added, M::mul(k, d), nrm);
                ++cnt;
            }
        }
    }
    if (cnt > 0) force = v_add<M>(force, v_div<M>(added, (float)cnt));
    return force;
}

// ---------------------------------------------------------------------------
// Grid helpers (compute.comp:217-252 splat, :258-293 gather).
// ---------------------------------------------------------------------------
struct Corners {
    float g[3];    // grid-space coordinates
    int lo[3];     // first corner per axis
    int cnt[3];    // 0, 1 or 2 corners per axis
    float flo[3];  // lo as a float (exact: small integers), so weights need no conversion
};

template <class M>
__device__ __forceinline__ Corners corners_of(const DevAsset& A, f3 p) {
    Corners C;
    const float pv[3] = {p.x, p.y, p.z};
    const int dim[3] = {A.nx, A.ny, A.nz};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        const float g = M::kExact ? M::div(M::sub(pv[ax], A.origin[ax]), A.h) : (pv[ax] - A.origin[ax]) * A.inv_h;
        float f = floorf(g);
        f = fminf(fmaxf(f, -2.0f), (float)dim[ax]);   // same corner set, defined conversion
        const int fi = (int)f;
        const int lo = max(fi, 0);
        const int hi = min(fi + 1, dim[ax] - 1);
        C.g[ax] = g;
        C.lo[ax] = lo;
        C.cnt[ax] = max(hi - lo + 1, 0);
        C.flo[ax] = fmaxf(f, 0.0f);
    }
    return C;
}

// clamp(1 - abs(g - a), 0, 1) for corner coordinate a (a float holding an integer)
template <class M>
__device__ __forceinline__ float tri_w(float g, float a) {
    return fminf(fmaxf(M::sub(1.0f, fabsf(M::sub(g, a))), 0.0f), 1.0f);
}

__device__ __forceinline__ long long fixed_of(float scale_times_x) {
    return (long long)__float2int_rz(scale_times_x);
}

// The four fixed-point contributions of one point to one corner, int(SCALE * w * v)
// (compute.comp:245-248).  Exact math keeps the oracle's scale * (w * v); fast
// math shares scale * w.  Every splat path calls this, so the box and the
// direct-atomic paths add identical integers.
template <class M>
__device__ __forceinline__ void corner_contribs(float scale, float w, f3 vel, int& q0, int& q1, int& q2, int& q3) {
    if (M::kExact) {
        q0 = __float2int_rz(M::mul(scale, M::mul(w, vel.x)));
        q1 = __float2int_rz(M::mul(scale, M::mul(w, vel.y)));
        q2 = __float2int_rz(M::mul(scale, M::mul(w, vel.z)));
    } else {
        const float sw = scale * w;
        q0 = __float2int_rz(sw * vel.x);
        q1 = __float2int_rz(sw * vel.y);
        q2 = __float2int_rz(sw * vel.z);
    }
    q3 = __float2int_rz(M::mul(scale, w));
}

__device__ __forceinline__ void red_add_s64(unsigned long long* p, long long v) {
    if (v != 0) atomicAdd(p, (unsigned long long)v);
}

// Splat one point: 4 x int64 atomics per touched corner, sums wrap-free.
// Only corners with x index in [xlo, xhi) are added.  (Inlined even where it
// is a rare fallback: a call costs spills around it at the call sites.)
template <class M>
__device__ __forceinline__ void splat_point(const DevAsset& A, f3 pos, f3 vel, int xlo = 0, int xhi = 0x7fffffff) {
    const Corners C = corners_of<M>(A, pos);
    const int nxny = A.nx * A.ny;
#pragma unroll
    for (int da = 0; da < 2; ++da) {
        if (da >= C.cnt[0]) continue;
        const int a = C.lo[0] + da;
        if (a < xlo || a >= xhi) continue;
        const float wx = tri_w<M>(C.g[0], C.flo[0] + (float)da);
#pragma unroll
        for (int db = 0; db < 2; ++db) {
            if (db >= C.cnt[1]) continue;
            const int b = C.lo[1] + db;
            const float wy = tri_w<M>(C.g[1], C.flo[1] + (float)db);
            const float wxy = M::mul(wx, wy);
#pragma unroll
            for (int dc = 0; dc < 2; ++dc) {
                if (dc >= C.cnt[2]) continue;
                const int c = C.lo[2] + dc;
                const float w = M::mul(wxy, tri_w<M>(C.g[2], C.flo[2] + (float)dc));
                unsigned long long* cell = A.grid + 4ull * (unsigned)(a + b * A.nx + c * nxny);
                int q0, q1, q2, q3;
                corner_contribs<M>(A.scale, w, vel, q0, q1, q2, q3);
                red_add_s64(cell + 0, q0);
                red_add_s64(cell + 1, q1);
                red_add_s64(cell + 2, q2);
                red_add_s64(cell + 3, q3);
            }
        }
    }
}

__device__ __forceinline__ long long grid_val(unsigned long long raw, bool wrap32) {
    return wrap32 ? (long long)(int)(unsigned)(raw & 0xffffffffull) : (long long)raw;
}

// One grid cell as the gather reads it: velocity sums as floats, the
// repulsion density rc = density / scale and rcp = 1 / density (rcp > 0
// exactly when the integer density is > 0).
struct CellF {
    float vx, vy, vz, rc, rcp;
};

// (float)x, rounded to nearest: the int32 conversion when x fits (the usual
// case; the same value), the int64 one otherwise.
__device__ __forceinline__ float i64_to_f32(long long x) {
    const int lo = (int)x;
    return (long long)lo == x ? __int2float_rn(lo) : __ll2float_rn(x);
}

template <class M>
__device__ __forceinline__ CellF cell_from_sums(long long vx, long long vy, long long vz, long long dens, float scale) {
    CellF c;
    c.vx = i64_to_f32(vx);
    c.vy = i64_to_f32(vy);
    c.vz = i64_to_f32(vz);
    const float fd = i64_to_f32(dens);
    c.rc = M::div(fd, scale);
    c.rcp = M::rcp(fd);
    return c;
}

template <class M>
__device__ __forceinline__ CellF cell_from_global(const DevAsset& A, const unsigned long long* grid, unsigned idx) {
    const ulonglong2* cell = reinterpret_cast<const ulonglong2*>(grid + 4ull * idx);
    const bool wrap = A.wrap32 != 0;
    const ulonglong2 zw = __ldcg(cell + 1);
    const long long dens = grid_val(zw.y, wrap);
    if (dens <= 0) return CellF{0.f, 0.f, 0.f, 0.f, 0.f};
    const ulonglong2 xy = __ldcg(cell);
    return cell_from_sums<M>(grid_val(xy.x, wrap), grid_val(xy.y, wrap), grid_val(zw.x, wrap), dens, A.scale);
}

// d(weight)/d(g) sign of corner a on one axis: -1 left of the point, +1 right
// of it, 0 outside the unit support (compute.comp repulsion extension).
template <class M>
__device__ __forceinline__ float grad_sign(float g, float a) {
    const float ga = M::sub(g, a);
    return fabsf(ga) < 1.0f ? (ga >= 0.0f ? -1.0f : 1.0f) : 0.0f;
}

// Gather + friction (+ repulsion) for one point (compute.comp:258-297);
// cell(a, b, c) returns the CellF of corner (a, b, c).  The per-axis weights,
// their pairwise products and the gradient signs are computed once per point;
// with signs in {-1, 0, 1} and weights >= 0, d * (w1 * w2) has the bits of
// (d * w1) * w2, so every corner term equals the oracle's.
template <class M, class CellFn>
__device__ __forceinline__ f3 gather_point(const DevAsset& A, float dt, f3 pos, f3 vel, const Corners& C, CellFn cell) {
    const bool rep = A.repulsion != 0.0f;
    float wxs[2], wys[2], wzs[2], sx[2] = {0.f, 0.f}, sy[2] = {0.f, 0.f}, sz[2] = {0.f, 0.f};
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        wxs[d] = tri_w<M>(C.g[0], C.flo[0] + (float)d);
        wys[d] = tri_w<M>(C.g[1], C.flo[1] + (float)d);
        wzs[d] = tri_w<M>(C.g[2], C.flo[2] + (float)d);
    }
    if (rep) {
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            sx[d] = grad_sign<M>(C.g[0], C.flo[0] + (float)d);
            sy[d] = grad_sign<M>(C.g[1], C.flo[1] + (float)d);
            sz[d] = grad_sign<M>(C.g[2], C.flo[2] + (float)d);
        }
    }
    f3 gv = {0.f, 0.f, 0.f};
    float rho = 0.f;
    f3 grad = {0.f, 0.f, 0.f};
    // Branch-free corner loop: a missing corner (past the grid) or an empty cell
    // contributes with weight 0 read from a valid cell of the point's range;
    // adding those +-0 terms leaves every sum's bits unchanged (no sum is ever
    // -0), so the result equals the oracle's, which skips them.
    if (C.cnt[0] > 0 && C.cnt[1] > 0 && C.cnt[2] > 0) {
#pragma unroll
        for (int da = 0; da < 2; ++da) {
            const bool ea = da < C.cnt[0];
            const int a = C.lo[0] + (ea ? da : 0);
#pragma unroll
            for (int db = 0; db < 2; ++db) {
                const bool eb = db < C.cnt[1];
                const int b = C.lo[1] + (eb ? db : 0);
                const float wxy = M::mul(wxs[da], wys[db]);
#pragma unroll
                for (int dc = 0; dc < 2; ++dc) {
                    const bool ec = dc < C.cnt[2];
                    const int c = C.lo[2] + (ec ? dc : 0);
                    const CellF cf = cell(a, b, c);
                    const bool live = ea && eb && ec && cf.rcp > 0.0f;
                    const float w = live ? M::mul(wxy, wzs[dc]) : 0.0f;
                    const float s = M::mul(w, cf.rcp);
                    gv = v_axpy<M>(gv, s, f3{cf.vx, cf.vy, cf.vz});
                    if (rep) {
                        const float rc = live ? cf.rc : 0.0f;
                        rho = M::madd(w, rc, rho);
                        const f3 dw = {M::mul(sx[da], M::mul(wys[db], wzs[dc])),
                                       M::mul(sy[db], M::mul(wxs[da], wzs[dc])), M::mul(sz[dc], wxy)};
                        grad = v_axpy<M>(grad, rc, dw);
                    }
                }
            }
        }
    }
    const float fr = A.friction;
    f3 out = v_axpy<M>(v_scale<M>(M::sub(1.0f, fr), vel), fr, gv);
    if (rep) {
        const float coef = M::div(M::mul(A.repulsion, M::div(A.h, dt)), fmaxf(rho, 1.0f));
        out = v_sub<M>(out, v_scale<M>(coef, grad));
    }
    return out;
}

// ---------------------------------------------------------------------------
// Fast-math gather.  A cell is 16 B: its mean velocity v_sum * (1/density)
// and rc = density / scale (all zero for an empty cell), and the trilinear
// sums are taken axis by axis: over z, then y, then x, so the eight corners
// cost 4 + 2 + 1 weighted float4 sums instead of eight weight products, and
// the repulsion gradient reuses the partial sums.  Same quantities as
// gather_point (compute.comp:280-297 plus the repulsion extension), in a
// different order of rounding.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float4 cellq_from_sums(long long vx, long long vy, long long vz, long long dens, float scale) {
    const float fd = i64_to_f32(dens);
    const float r = FastMath::rcp(fd);
    return make_float4(i64_to_f32(vx) * r, i64_to_f32(vy) * r, i64_to_f32(vz) * r, FastMath::div(fd, scale));
}

__device__ __forceinline__ float4 cellq_from_global(const DevAsset& A, const unsigned long long* grid, unsigned idx) {
    const ulonglong2* cell = reinterpret_cast<const ulonglong2*>(grid + 4ull * idx);
    const bool wrap = A.wrap32 != 0;
    const ulonglong2 zw = __ldcg(cell + 1);
    const long long dens = grid_val(zw.y, wrap);
    if (dens <= 0) return make_float4(0.f, 0.f, 0.f, 0.f);
    const ulonglong2 xy = __ldcg(cell);
    return cellq_from_sums(grid_val(xy.x, wrap), grid_val(xy.y, wrap), grid_val(zw.x, wrap), dens, A.scale);
}

__device__ __forceinline__ float4 f4_axpy(float4 acc, float w, float4 q) {
    return make_float4(fmaf(w, q.x, acc.x), fmaf(w, q.y, acc.y), fmaf(w, q.z, acc.z), fmaf(w, q.w, acc.w));
}
__device__ __forceinline__ float4 f4_lerp(float w0, float4 q0, float w1, float4 q1) {
    return f4_axpy(make_float4(w0 * q0.x, w0 * q0.y, w0 * q0.z, w0 * q0.w), w1, q1);
}

// cellq(i) returns the 16-B cell at linear index i of the array it reads;
// base is corner (lo, lo, lo)'s index and sy, sz the array's row and slab
// pitches.  A corner past the grid gets weight and gradient sign 0 and reads
// a valid cell of the point's own range.
template <class CellFn>
__device__ __forceinline__ f3 gather_point_fast(const DevAsset& A, float dt, f3 vel, const Corners& C, int base, int sy,
                                                int sz, CellFn cellq) {
    using M = FastMath;
    const bool rep = A.repulsion != 0.0f;
    f3 gv = {0.f, 0.f, 0.f}, grad = {0.f, 0.f, 0.f};
    float rho = 0.f;
    if (C.cnt[0] > 0 && C.cnt[1] > 0 && C.cnt[2] > 0) {
        float w[3][2];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax)
#pragma unroll
            for (int d = 0; d < 2; ++d)
                w[ax][d] = d < C.cnt[ax] ? tri_w<M>(C.g[ax], C.flo[ax] + (float)d) : 0.f;
        const int ox = C.cnt[0] > 1 ? 1 : 0, oy = C.cnt[1] > 1 ? sy : 0, oz = C.cnt[2] > 1 ? sz : 0;
        // corner (a, b, c): z sums Zab first, then y sums Y[a], then the x sum; the
        // repulsion gradient's y and z terms (ty over a and c, tz over a and b)
        // accumulate as the corners stream by
        float4 Y[2];
        float ty[2] = {0.f, 0.f}, tz[2] = {0.f, 0.f};
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                const int i0 = base + (a ? ox : 0) + (b ? oy : 0);
                const float4 q0 = cellq(i0);
                const float4 q1 = cellq(i0 + oz);
                const float4 Zab = f4_lerp(w[2][0], q0, w[2][1], q1);
                Y[a] = b == 0 ? make_float4(w[1][0] * Zab.x, w[1][0] * Zab.y, w[1][0] * Zab.z, w[1][0] * Zab.w)
                              : f4_axpy(Y[a], w[1][1], Zab);
                if (rep) {
                    ty[b] = fmaf(w[0][a], Zab.w, ty[b]);
                    const float wab = w[0][a] * w[1][b];
                    tz[0] = fmaf(wab, q0.w, tz[0]);
                    tz[1] = fmaf(wab, q1.w, tz[1]);
                }
            }
        const float4 X = f4_lerp(w[0][0], Y[0], w[0][1], Y[1]);
        gv = f3{X.x, X.y, X.z};
        if (rep) {
            float sg[3][2];   // d(weight)/d(g) signs; 0 for a corner past the grid
#pragma unroll
            for (int ax = 0; ax < 3; ++ax)
#pragma unroll
                for (int d = 0; d < 2; ++d)
                    sg[ax][d] = d < C.cnt[ax] ? grad_sign<M>(C.g[ax], C.flo[ax] + (float)d) : 0.f;
            rho = X.w;
            grad.x = fmaf(sg[0][1], Y[1].w, sg[0][0] * Y[0].w);
            grad.y = fmaf(sg[1][1], ty[1], sg[1][0] * ty[0]);
            grad.z = fmaf(sg[2][1], tz[1], sg[2][0] * tz[0]);
        }
    }
    const float fr = A.friction;
    f3 out = v_axpy<M>(v_scale<M>(M::sub(1.0f, fr), vel), fr, gv);
    if (rep) {
        const float coef = M::div(M::mul(A.repulsion, M::div(A.h, dt)), fmaxf(rho, 1.0f));
        out = v_sub<M>(out, v_scale<M>(coef, grad));
    }
    return out;
}

// head * (p, 1) for a row-major 3 x 4 affine head: ((h0 x + h1 y) + h2 z) + h3 per row.
template <class M>
__device__ __forceinline__ f3 head_point(const float (&h)[12], f3 p) {
    f3 o;
    o.x = M::add(M::madd(h[2], p.z, M::madd(h[1], p.y, M::mul(h[0], p.x))), h[3]);
    o.y = M::add(M::madd(h[6], p.z, M::madd(h[5], p.y, M::mul(h[4], p.x))), h[7]);
    o.z = M::add(M::madd(h[10], p.z, M::madd(h[9], p.y, M::mul(h[8], p.x))), h[11]);
    return o;
}

// ---------------------------------------------------------------------------
// Phase A for one strand group.
//   A warp holds S = 32/L strands; the L lanes of a strand hold its points in
//   an interleaved order (lane l holds points l, l+L, l+2L, ...), so each
//   16-B load/store instruction covers 16*L contiguous bytes per strand.
//   The FTL chain (sequential along the strand) runs redundantly in every lane
//   of the strand with the predicted points broadcast by shuffles; each lane
//   keeps the results for its own points.
//   NFIX > 0 fixes the point count at compile time; NFIX == 0 reads it from
//   the asset (any n <= RVH_MAX_POINTS).
// All lanes of the warp must call this (shuffles); `valid` masks the work.
// ---------------------------------------------------------------------------
template <int NFIX, int L>
struct PhaseA {
    static constexpr int NMAX = NFIX > 0 ? NFIX : RVH_MAX_POINTS;
    static constexpr int K = (NMAX + L - 1) / L;
    // point held in slot k of lane l, and the (lane, slot) holding point i
    static __device__ __forceinline__ int point(int l, int k) { return k * L + l; }
    static __device__ __forceinline__ int owner(int i) { return i % L; }
    static __device__ __forceinline__ int slot(int i) { return i / L; }
};

// Loads the lane's points (positions and velocities) of one strand; bit k of
// the result is set when point k exists and is not the root.
template <int NFIX, int L>
__device__ __forceinline__ unsigned load_points(const DevAsset& A, int strand, bool valid,
                                                f3 (&x)[PhaseA<NFIX, L>::K], f3 (&v)[PhaseA<NFIX, L>::K]) {
    constexpr int K = PhaseA<NFIX, L>::K;
    const int n = NFIX > 0 ? NFIX : A.n_points;
    const int l = (threadIdx.x & 31) % L;
    const float4* rec = A.strands + (size_t)(valid ? strand : 0) * (3 * n);
    unsigned mask = 0u;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = PhaseA<NFIX, L>::point(l, k);
        if (valid && i < n) {
            x[k] = xyz(ld_cg(rec + i));
            v[k] = xyz(ld_cg(rec + n + i));
            if (i >= 1) mask |= 1u << k;
        } else {
            x[k] = f3{0.f, 0.f, 0.f};
            v[k] = f3{0.f, 0.f, 0.f};
        }
    }
    return mask;
}

// Computes loops 1-2 for the lane's points (x, v as loaded), stores x', v,
// corr, and returns the splat inputs: xo/vo for the lane's points, bit k of
// the result set when point k is splatted (valid strand, 1 <= i < n).
template <int NFIX, int L, class M>
__device__ __forceinline__ unsigned strand_phase_a(const DevAsset& A, int strand, bool valid,
                                                   const f3 (&x)[PhaseA<NFIX, L>::K], const f3 (&vel_in)[PhaseA<NFIX, L>::K],
                                                   f3 (&xo)[PhaseA<NFIX, L>::K], f3 (&vo)[PhaseA<NFIX, L>::K]) {
    constexpr int NMAX = PhaseA<NFIX, L>::NMAX;
    constexpr int K = PhaseA<NFIX, L>::K;
    const int n = NFIX > 0 ? NFIX : A.n_points;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int l = lane % L;
    const int base = lane - l;
    float4* rec = A.strands + (size_t)(valid ? strand : 0) * (3 * n);

    f3 p[K], xn[K];
#pragma unroll
    for (int k = 0; k < K; ++k) xn[k] = x[k];  // the root (i == 0) keeps its position
    const float dt = A.dt;
    const float r = valid ? A.rest[strand] : 0.f;
    f3 f0 = v_add<M>(f3{A.gravity[0], A.gravity[1], A.gravity[2]}, f3{A.wind[0], A.wind[1], A.wind[2]});
    if (A.strand_wind != nullptr && valid) f0 = v_add<M>(f0, xyz(A.strand_wind[strand]));
    const float dt2 = M::mul(dt, dt);

    // loop 1, independent part: force and predicted position of each point
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = PhaseA<NFIX, L>::point(l, k);
        f3 force = f0;
        if (valid && i >= 1 && i < n) force = collide_force<M>(A, x[k], force);
        const f3 v = vel_in[k];
        // predictedPos = currentPos + dt * currentVel + dt * dt * force   (compute.comp:187)
        p[k] = v_axpy<M>(v_axpy<M>(x[k], dt, v), dt2, force);
    }

    // loop 1, sequential part: FTL, newPos = parent + radius * normalize(pred - parent)
    f3 par;
    if (L == 1) {
        par = x[0];
    } else {
        par.x = __shfl_sync(FULL, x[0].x, base);
        par.y = __shfl_sync(FULL, x[0].y, base);
        par.z = __shfl_sync(FULL, x[0].z, base);
    }
    const bool moving = A.root_rest != nullptr;
    if (moving) {
        // kinematic head: the root follows it (every lane of the strand computes the same root)
        const f3 r0 = valid ? xyz(A.root_rest[strand]) : f3{0.f, 0.f, 0.f};
        par = head_point<M>(A.head, r0);
        if (l == 0) xn[0] = par;
    }
    if constexpr (L > 1 && K > 1) {
        // the chain over slot k in a rolled loop (the current slot is p[0] and xn[0],
        // rotated after each pass, back in order after K), the L owners of a slot unrolled:
        // a quarter of the code of a fully unrolled chain at n = 32, the same operations
#pragma unroll 1
        for (int k = 0; k < K; ++k) {
#pragma unroll
            for (int o = 0; o < L; ++o) {
                const int i = k * L + o;
                if (i >= n) break;   // n is uniform across the warp
                if (i == 0) continue;   // the root
                f3 pi;
                pi.x = __shfl_sync(FULL, p[0].x, base + o);
                pi.y = __shfl_sync(FULL, p[0].y, base + o);
                pi.z = __shfl_sync(FULL, p[0].z, base + o);
                const f3 dir = v_normalize<M>(v_sub<M>(pi, par));
                par = v_axpy<M>(par, r, dir);
                if (l == o) xn[0] = par;
            }
            const f3 tp = p[0], tx = xn[0];
#pragma unroll
            for (int q = 0; q + 1 < K; ++q) {
                p[q] = p[q + 1];
                xn[q] = xn[q + 1];
            }
            p[K - 1] = tp;
            xn[K - 1] = tx;
        }
    } else {
#pragma unroll
    for (int i = 1; i < NMAX; ++i) {
        if (NFIX == 0 && i >= n) break;  // n is uniform across the warp
        const int k = PhaseA<NFIX, L>::slot(i), own = PhaseA<NFIX, L>::owner(i);
        f3 pi;
        if (L == 1) {
            pi = p[k];
        } else {
            pi.x = __shfl_sync(FULL, p[k].x, base + own);
            pi.y = __shfl_sync(FULL, p[k].y, base + own);
            pi.z = __shfl_sync(FULL, p[k].z, base + own);
        }
        const f3 dir = v_normalize<M>(v_sub<M>(pi, par));
        par = v_axpy<M>(par, r, dir);
        if (L == 1 || l == own) xn[k] = par;
    }
    }

    // velocity, clamp and correction vector (compute.comp:195-201)
    f3 vel[K], cor[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const f3 newVel = v_div<M>(v_sub<M>(xn[k], x[k]), dt);
        f3 v = v_scale<M>(A.damping, newVel);
        if (v_len<M>(v) > A.vmax) v = v_scale<M>(A.vmax, v_normalize<M>(v));
        vel[k] = v;
        cor[k] = v_scale<M>(A.dftl, v_sub<M>(xn[k], p[k]));
    }

    // loop 2: v_i -= corr_{i+1} / dt for i < n-1 (compute.comp:213-215)
    // point i+1 is the same slot of the next lane, or the next slot of lane 0
#pragma unroll
    for (int k = 0; k < K; ++k) {
        f3 cn;
        if (L == 1) {
            cn = (k + 1 < K) ? cor[k + 1] : f3{0.f, 0.f, 0.f};
        } else {
            f3 same, wrap;
            same.x = __shfl_sync(FULL, cor[k].x, (lane + 1) & 31);
            same.y = __shfl_sync(FULL, cor[k].y, (lane + 1) & 31);
            same.z = __shfl_sync(FULL, cor[k].z, (lane + 1) & 31);
            const f3 nxt = (k + 1 < K) ? cor[k + 1] : f3{0.f, 0.f, 0.f};
            wrap.x = __shfl_sync(FULL, nxt.x, base);
            wrap.y = __shfl_sync(FULL, nxt.y, base);
            wrap.z = __shfl_sync(FULL, nxt.z, base);
            cn = (l + 1 < L) ? same : wrap;
        }
        const int i = PhaseA<NFIX, L>::point(l, k);
        if (i >= 1 && i < n - 1) vel[k] = v_sub<M>(vel[k], v_div<M>(cn, dt));
    }

    // store x', v, corr for points 1..n-1 (the root is written only when a head moves it)
    if (moving && valid && l == 0) st_f4(rec, xn[0], 1.0f);
    if (A.pos_xyz != nullptr && valid) {   // every point's position, the root included
        float* o = A.pos_xyz + 3 * ((size_t)strand * n);
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int i = PhaseA<NFIX, L>::point(l, k);
            if (i < n) {
                o[3 * i] = xn[k].x;
                o[3 * i + 1] = xn[k].y;
                o[3 * i + 2] = xn[k].z;
            }
        }
    }
    unsigned mask = 0u;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = PhaseA<NFIX, L>::point(l, k);
        if (valid && i >= 1 && i < n) {
            st_f4(rec + i, xn[k], 1.0f);
            st_f4(rec + n + i, vel[k], 0.0f);
            st_f4(rec + 2 * n + i, cor[k], 0.0f);
            mask |= 1u << k;
        }
        xo[k] = xn[k];
        vo[k] = vel[k];
    }
    return mask;
}

}  // namespace rvh
