// rvh_kernels.cuh — kernel templates of the hair step.
//
//   k_plain_a / k_plain_b : one asset per launch sequence (the drop-in for one
//                           Renderer::Frame() compute submit, src/Renderer.cpp:
//                           2063-2071: clear grid, dispatch).
//   k_batch               : every asset of a batch in ONE persistent launch.
//                           CTAs pull work items (grid clears, phase-A strand
//                           tiles, phase-B point tiles) from a queue in order; a
//                           phase-B tile waits (bounded) on its asset's count of
//                           finished phase-A tiles.  Items are fetched in queue
//                           order and every wait is on items earlier in the
//                           queue, so the launch makes progress whatever the
//                           number of co-resident CTAs.
#pragma once

#include "rvh_device.cuh"

namespace rvh {

constexpr int kThreads = 256;          // CTA size of every step kernel
constexpr int kWarps = kThreads / 32;
constexpr int kSmemBytes = 72 * 1024;  // dynamic shared memory per CTA (grid boxes)
constexpr int kMinCtasPerSm = 3;       // 3 x 72 KB of boxes and <= 80 registers per thread per SM
constexpr int kUnionRounds = 4;        // rounds sharing one gather box and one splat box
constexpr int kBoxCellsA = kSmemBytes / 16;   // phase A: 4 x int32 partial sums per cell
// gather boxes: exact math keeps CellF (float4 + rcp, 20 B), fast math a 16-B normalised cell
template <class M> constexpr int box_cells_b() { return M::kExact ? kSmemBytes / 20 : kSmemBytes / 16; }
constexpr int kTileB = 2048;           // points per phase-B tile
constexpr int kPtsB = kTileB / kThreads;

enum : int32_t { ITEM_CLEAR = 0, ITEM_A = 1, ITEM_B = 2 };

struct WorkItem {
    int32_t kind;
    int32_t asset;
    int32_t begin;   // strands (A, B) or 16-B grid chunks (CLEAR)
    int32_t end;
};

struct BatchDev {
    const DevAsset* assets;
    const WorkItem* items;
    int32_t n_items;
    uint32_t spin_limit;        // bounded wait of a phase-B tile (iterations of ~256 ns)
    int32_t prefetch;           // nonzero: ask L2 for the next phase-A item's strands (large items)
    int32_t count_clears;       // nonzero (several steps per launch): clears count in done_a; otherwise
                                // they do not, as a phase-B tile's wait counts phase-A tiles only
    unsigned* head;             // next item (reset to 0 before every launch)
    unsigned* done_a;           // per entry: finished phase-A tiles (and clears, with count_clears;
                                // reset before every launch)
    const unsigned* need_a;     // per entry: phase-A tiles in this launch (plus its clears when a
                                // later step of the asset waits on them)
    int* error;                 // nonzero: a wait gave up (RVH_ERR_TIMEOUT)
    unsigned* stats;            // [0] phase-A rounds splatted through the shared box, [1] directly;
                                // [2] phase-B tiles gathered from the box, [3] directly
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Unsigned division by a runtime divisor d via a multiply-high: with
// m = floor((2^32 - 1) / d) + 1, umulhi(c, m) = floor(c / d) whenever
// c * d < 2^32 (box cells and tile points here stay below 2^16).
struct FastDiv {
    unsigned m, d;
    __device__ __forceinline__ explicit FastDiv(unsigned dd) : m(dd > 1 ? 0xffffffffu / dd + 1u : 0u), d(dd) {}
    __device__ __forceinline__ unsigned div(unsigned c) const { return d > 1 ? __umulhi(c, m) : c; }
};

// ---- shared-memory grid boxes ----------------------------------------------------
// A CTA's points touch a compact block of grid cells.  Phase A accumulates its
// splat in that box with shared-memory int32 atomics and flushes each touched
// cell once with int64 global atomics; phase B copies its box once from the
// grid and gathers from shared memory.  Integer sums are order independent, so
// both give exactly the bits of the direct global-atomic path.
struct BoxShared {
    int lo[3];
    int hi[3];
    unsigned vabs;   // max |v| component of the round's points (float bits)
    int npts;        // points with at least one corner
};

__device__ __forceinline__ void box_reset(BoxShared& S) {
    if (threadIdx.x == 0) {
        for (int a = 0; a < 3; ++a) {
            S.lo[a] = 0x7fffffff;
            S.hi[a] = -0x7fffffff - 1;
        }
        S.vabs = 0u;
        S.npts = 0;
    }
}

__device__ __forceinline__ void box_reduce(BoxShared& S, const int (&lmin)[3], const int (&lmax)[3], unsigned vabs,
                                           int np) {
    const unsigned FULL = 0xffffffffu;
    int mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        mn[a] = __reduce_min_sync(FULL, lmin[a]);
        mx[a] = __reduce_max_sync(FULL, lmax[a]);
    }
    const unsigned va = __reduce_max_sync(FULL, vabs);
    const int n = (int)__reduce_add_sync(FULL, (unsigned)np);
    if ((threadIdx.x & 31) == 0 && n > 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(&S.lo[a], mn[a]);
            atomicMax(&S.hi[a], mx[a]);
        }
        atomicMax(&S.vabs, va);
        atomicAdd(&S.npts, n);
    }
}

__device__ __forceinline__ void bounds_add(const Corners& C, int (&lmin)[3], int (&lmax)[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lmin[a] = min(lmin[a], C.lo[a]);
        lmax[a] = max(lmax[a], C.lo[a] + C.cnt[a] - 1);
    }
}

__device__ __forceinline__ bool has_corners(const Corners& C) { return C.cnt[0] > 0 && C.cnt[1] > 0 && C.cnt[2] > 0; }

// Box bounds from the lane's position extremes.  g = (p - o)/h and the corner
// range [max(floor g, 0), min(floor g + 1, dim - 1)] are monotone in p, so the
// corners of the extremes bound the corners of every point in between; lanes
// without points leave the bounds empty.
template <class M>
__device__ __forceinline__ void bounds_of_extremes(const DevAsset& A, f3 pmin, f3 pmax, int (&lmin)[3], int (&lmax)[3]) {
    const Corners C0 = corners_of<M>(A, pmin), C1 = corners_of<M>(A, pmax);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lmin[a] = C0.lo[a];
        lmax[a] = max(C1.lo[a] + C1.cnt[a] - 1, C0.lo[a]);
    }
}

// Shape of a box in shared memory: cells [lo, lo + ext) of the grid, x
// fastest, with odd row and slab pitches (py = ext_x | 1, pz = (py * ext_y) | 1)
// so that cells one row or one slab apart fall in different banks; the padding
// cells are never touched by a point.  vol counts the padded cells.
struct BoxGeom {
    int lo[3];
    int ext[3];
    int py, pz;
    long long vol;
    __device__ __forceinline__ int offset(int a, int b, int c) const {
        return (a - lo[0]) + py * (b - lo[1]) + pz * (c - lo[2]);
    }
};

__device__ __forceinline__ BoxGeom box_geom(const BoxShared& S) {
    BoxGeom G;
    long long e[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        G.lo[a] = S.lo[a];
        e[a] = (long long)S.hi[a] - S.lo[a] + 1;   // <= 0 for an empty box
        G.ext[a] = (int)(e[a] > 0 ? (e[a] < 0x40000000LL ? e[a] : 0x40000000LL) : 0);
    }
    const long long py = e[0] > 0 ? (e[0] | 1) : 1;
    const long long pz = (py * (e[1] > 0 ? e[1] : 0)) | 1;
    G.vol = (e[0] > 0 && e[1] > 0 && e[2] > 0) ? pz * e[2] : (1LL << 62);   // an empty box is never used
    G.py = (int)(py < 0x40000000LL ? py : 0x40000000LL);
    G.pz = (int)(pz < 0x40000000LL ? pz : 0x40000000LL);
    return G;
}

// Grid coordinates of padded box cell c, false for a padding cell.
struct BoxWalk {
    FastDiv dy, dz;
    __device__ __forceinline__ explicit BoxWalk(const BoxGeom& G) : dy((unsigned)G.py), dz((unsigned)G.pz) {}
    __device__ __forceinline__ bool cell(const BoxGeom& G, int c, int& a, int& b, int& cc) const {
        const int qz = (int)dz.div((unsigned)c), rz = c - qz * G.pz;
        const int qy = (int)dy.div((unsigned)rz), rx = rz - qy * G.py;
        a = G.lo[0] + rx;
        b = G.lo[1] + qy;
        cc = G.lo[2] + qz;
        return rx < G.ext[0] && qy < G.ext[1];
    }
};

// Splat one point into the shared box (int32 partial sums): its corners with
// x index in [G.lo[0], G.lo[0] + G.ext[0]).  The box holds four component
// arrays (vx, vy, vz, density) kBoxCellsA cells apart, so each component's
// address is the cell's plus a constant, and one component's atomics from a
// warp spread over the banks.  The six trilinear weights of a point are
// computed once.  Exact math keeps the oracle's int(scale * (w * v)); fast
// math shares scale * w.
// Per-lane corner order (integer sums do not depend on it): in step j lane l
// adds corner j ^ (l mod 8), so lanes whose points share a cell hit different
// corners in the same instruction.  The order is set once per point by
// swapping the two corners of each axis whose bit is set in l mod 8; every
// step then has compile-time corner indices, and each corner's weight is
// still (wx * wy) * wz.
template <int L, class M>
__device__ __forceinline__ void splat_point_box(const DevAsset& A, const Corners& C, f3 vel, int* box, const BoxGeom& G) {
    // the corners inside the slab: x in [dlo, dhi] of {0, 1}; y, z in [0, cnt - 1]
    const int x0 = G.lo[0] - C.lo[0];
    const int dlo = max(0, x0), dhi = min(C.cnt[0], x0 + G.ext[0]) - 1;
    if (dhi < dlo || C.cnt[1] <= 0 || C.cnt[2] <= 0) return;   // no corner in this slab
    // Branch-free corner loop: a missing corner gets weight 0 at a valid cell
    // of the point's own range, so its atomics add 0 (integer sums are unchanged).
    float w[3][2];
    int o[3][2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        const bool ex = d >= dlo && d <= dhi, ey = d < C.cnt[1], ez = d < C.cnt[2];
        w[0][d] = ex ? tri_w<M>(C.g[0], C.flo[0] + (float)d) : 0.f;
        w[1][d] = ey ? tri_w<M>(C.g[1], C.flo[1] + (float)d) : 0.f;
        w[2][d] = ez ? tri_w<M>(C.g[2], C.flo[2] + (float)d) : 0.f;
        o[0][d] = ex ? d : dlo;
        o[1][d] = (ey ? d : 0) * G.py;
        o[2][d] = (ez ? d : 0) * G.pz;
    }
    const int rot = (int)threadIdx.x & 7;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        const bool sw = (rot >> ax) & 1;
        const float w0 = w[ax][0], w1 = w[ax][1];
        const int o0 = o[ax][0], o1 = o[ax][1];
        w[ax][0] = sw ? w1 : w0;
        w[ax][1] = sw ? w0 : w1;
        o[ax][0] = sw ? o1 : o0;
        o[ax][1] = sw ? o0 : o1;
    }
    int* const b0 = box + G.offset(C.lo[0], C.lo[1], C.lo[2]);
#pragma unroll
    for (int da = 0; da < 2; ++da) {
#pragma unroll
        for (int db = 0; db < 2; ++db) {
            const float wxy = M::mul(w[0][da], w[1][db]);
            int* const bxy = b0 + (o[0][da] + o[1][db]);
#pragma unroll
            for (int dc = 0; dc < 2; ++dc) {
                int* cell = bxy + o[2][dc];
                int q0, q1, q2, q3;
                corner_contribs<M>(A.scale, M::mul(wxy, w[2][dc]), vel, q0, q1, q2, q3);
                atomicAdd(cell, q0);
                atomicAdd(cell + kBoxCellsA, q1);
                atomicAdd(cell + 2 * kBoxCellsA, q2);
                atomicAdd(reinterpret_cast<unsigned*>(cell + 3 * kBoxCellsA), (unsigned)q3);
            }
        }
    }
}

// Widest x slab of box G whose padded cells fit `cap` cells (0: none fits).
__device__ __forceinline__ int slab_width(const BoxGeom& G, int cap) {
    if (G.vol <= cap) return G.ext[0];
    // vol(w) = (((w | 1) * e1) | 1) * e2 <= ((w + 1) * e1 + 1) * e2
    const long long per = cap / G.ext[2] - 1;
    const long long w = per / G.ext[1] - 1;
    return (int)(w > 0 ? (w < G.ext[0] ? w : G.ext[0]) : 0);
}

// Bounds, |v| and count of a lane's points, accumulated one point at a time.
struct LaneBounds {
    f3 pmin = {3.0e38f, 3.0e38f, 3.0e38f}, pmax = {-3.0e38f, -3.0e38f, -3.0e38f};
    float vab = 0.f;
    int np = 0;
    __device__ __forceinline__ void add(f3 p) {
        pmin = f3{fminf(pmin.x, p.x), fminf(pmin.y, p.y), fminf(pmin.z, p.z)};
        pmax = f3{fmaxf(pmax.x, p.x), fmaxf(pmax.y, p.y), fmaxf(pmax.z, p.z)};
        ++np;
    }
    __device__ __forceinline__ void add_v(f3 v) { vab = fmaxf(vab, fmaxf(fabsf(v.x), fmaxf(fabsf(v.y), fabsf(v.z)))); }
    // the CTA's cell box of every lane's points into S (all threads call it)
    template <class M>
    __device__ __forceinline__ void reduce(const DevAsset& A, BoxShared& S) const {
        int lmin[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, lmax[3] = {-0x7fffffff - 1, -0x7fffffff - 1, -0x7fffffff - 1};
        if (np > 0) bounds_of_extremes<M>(A, pmin, pmax, lmin, lmax);
        box_reset(S);
        __syncthreads();
        box_reduce(S, lmin, lmax, __float_as_uint(vab), np);
        __syncthreads();
    }
};

// Splats the CTA's points into A.grid; every thread calls it after
// LaneBounds::reduce.  visit(f) calls f(position, velocity) for each of the
// lane's points.  The cell box is accumulated in shared memory in x slabs that
// fit (one slab in almost every round), each flushed once with int64 global
// atomics.  Velocity partials are int32, densities uint32 (npts * scale < 4e9
// keeps them exact).  A slab falls back to direct global atomics when its
// velocity partials cannot be proven free of overflow (|partial| <= vmax *
// (density + npts) since |int(s w v)| <= vmax * (int(s w) + 1)); the whole
// round does when not even a one-cell-wide slab fits or npts * scale >= 4e9.
template <int L, class M, class Visit>
__device__ __forceinline__ void splat_points(const DevAsset& A, int* box, BoxShared& S, unsigned* stats, Visit visit) {
    const int npts = S.npts;
    if (npts > 0) {
        const BoxGeom G = box_geom(S);
        // density partials are unsigned (every int(s w) >= 0): exact below 2^32
        const int w = (float)npts * A.scale < 4.0e9f ? slab_width(G, kBoxCellsA) : 0;
        const float vmax = __uint_as_float(S.vabs);
        const int nxny = A.nx * A.ny;
        bool all_box = w > 0;
        for (int x0 = G.lo[0]; w > 0 && x0 < G.lo[0] + G.ext[0]; x0 += w) {
            BoxGeom P = G;   // the slab [x0, x0 + w) of G
            P.lo[0] = x0;
            P.ext[0] = min(w, G.lo[0] + G.ext[0] - x0);
            P.py = P.ext[0] | 1;
            P.pz = (P.py * P.ext[1]) | 1;
            const int nv = P.pz * P.ext[2];
            int4* b4 = reinterpret_cast<int4*>(box);   // four component arrays, kBoxCellsA cells apart
            constexpr int kQ = kBoxCellsA / 4;
            for (int c = threadIdx.x; c < (nv + 3) / 4; c += kThreads) {
                b4[c] = make_int4(0, 0, 0, 0);
                b4[kQ + c] = make_int4(0, 0, 0, 0);
                b4[2 * kQ + c] = make_int4(0, 0, 0, 0);
                b4[3 * kQ + c] = make_int4(0, 0, 0, 0);
            }
            __syncthreads();
            visit([&](f3 p, f3 v) { splat_point_box<L, M>(A, corners_of<M>(A, p), v, box, P); });
            __syncthreads();
            bool ok = true;
            for (int c = threadIdx.x; c < nv; c += kThreads)
                ok = ok && vmax * ((float)(unsigned)box[3 * kBoxCellsA + c] + (float)npts) < 2.0e9f;
            if (__syncthreads_and(ok)) {
                const BoxWalk W(P);
                for (int c = threadIdx.x; c < nv; c += kThreads) {
                    const int4 v = make_int4(box[c], box[kBoxCellsA + c], box[2 * kBoxCellsA + c], box[3 * kBoxCellsA + c]);
                    if (!(v.x | v.y | v.z | v.w)) continue;   // untouched (padding cells always are)
                    int a, b, cc;
                    W.cell(P, c, a, b, cc);
                    unsigned long long* cell = A.grid + 4ull * (unsigned)(a + b * A.nx + cc * nxny);
                    red_add_s64(cell + 0, v.x);
                    red_add_s64(cell + 1, v.y);
                    red_add_s64(cell + 2, v.z);
                    red_add_s64(cell + 3, (long long)(unsigned)v.w);
                }
            } else {
                all_box = false;
                const int x1 = x0 + P.ext[0];
                visit([&](f3 p, f3 v) { splat_point<M>(A, p, v, x0, x1); });
            }
            __syncthreads();   // the box is cleared again by the next slab
        }
        if (w == 0) visit([&](f3 p, f3 v) { splat_point<M>(A, p, v); });
        if (stats && threadIdx.x == 0) atomicAdd(stats + (all_box ? 0 : 1), 1u);
    }
    __syncthreads();  // every read of S and of the box is done before the next round resets them
}

// Rolled loops over a lane's K register-held points: the body is emitted once
// and the point arrays rotate one slot per iteration (back in order after K),
// so the large splat and gather bodies are not unrolled K times (instruction
// cache).  kRolledPoints = false unrolls them instead.
constexpr bool kRolledPoints = true;

template <int K>
__device__ __forceinline__ void rotate_points(f3 (&a)[K]) {
    const f3 t = a[0];
#pragma unroll
    for (int k = 0; k + 1 < K; ++k) a[k] = a[k + 1];
    a[K - 1] = t;
}

// f(x[k], v[k]) for every k with mask bit k set; v may be updated by f.
template <int K, class F>
__device__ __forceinline__ void for_lane_points(f3 (&x)[K], f3 (&v)[K], unsigned mask, F&& f) {
    if (kRolledPoints && K > 1) {
        unsigned m = mask;
#pragma unroll 1
        for (int k = 0; k < K; ++k) {
            if (m & 1u) f(x[0], v[0]);
            rotate_points(x);
            rotate_points(v);
            m = (m >> 1) | ((m & 1u) << (K - 1));
        }
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if ((mask >> k) & 1u) f(x[k], v[k]);
    }
}

// Copies the box's cells of grid G into shared memory: exact math as CellF
// (float4 {vx, vy, vz, rc} at bf[c], rcp at br[c]), fast math as the 16-B
// normalised cell at bf[c].  Padding cells are skipped, and so are cells past
// the grid's last layer: a point beyond the grid has no corner on that axis
// but still widens the box there.
template <class M>
__device__ __forceinline__ void load_gather_box(const DevAsset& A, const unsigned long long* grid, const BoxGeom& G,
                                                float4* bf, float* br) {
    const int nxny = A.nx * A.ny;
    const int vol = (int)G.vol;
    const BoxWalk W(G);
    for (int c = threadIdx.x; c < vol; c += kThreads) {
        int a, b, cc;
        if (!W.cell(G, c, a, b, cc) || a >= A.nx || b >= A.ny || cc >= A.nz) continue;
        const unsigned idx = (unsigned)(a + b * A.nx + cc * nxny);
        if constexpr (M::kExact) {
            const CellF cf = cell_from_global<M>(A, grid, idx);
            bf[c] = make_float4(cf.vx, cf.vy, cf.vz, cf.rc);
            br[c] = cf.rcp;
        } else {
            bf[c] = cellq_from_global(A, grid, idx);
        }
    }
}

// Loop 3 for one point read straight from the grid (the rare fallback of the
// gather boxes).
template <class M>
__device__ __forceinline__ f3 gather_point_direct(const DevAsset& A, const unsigned long long* grid, float dt, f3 x, f3 v) {
    const int nxny = A.nx * A.ny;
    if constexpr (M::kExact) {
        return gather_point<M>(A, dt, x, v, corners_of<M>(A, x), [&](int a, int b, int c) {
            return cell_from_global<M>(A, grid, (unsigned)(a + b * A.nx + c * nxny));
        });
    } else {
        const Corners C = corners_of<M>(A, x);
        return gather_point_fast(A, dt, v, C, C.lo[0] + C.lo[1] * A.nx + C.lo[2] * nxny, A.nx, nxny,
                                 [&](int i) { return cellq_from_global(A, grid, (unsigned)i); });
    }
}

// The CTA's gather box over grid `grid` (after LaneBounds::reduce of the
// points to gather): loaded into shared memory when it fits, else the gather
// reads the grid directly.  gather(x, v, dt) then returns loop 3's velocity.
// The box geometry lives in shared memory (G), so holding the object across a
// group of rounds costs no registers.  A null grid builds an unused object (no
// synchronisation, no loads).
struct GatherShared {
    BoxGeom G;
    int use;
};

template <class M>
struct GatherBox {
    const DevAsset& A;
    const unsigned long long* grid;
    const GatherShared& GS;
    unsigned char* smem;
    static constexpr int kCap = box_cells_b<M>();
    __device__ __forceinline__ GatherBox(const DevAsset& a, const unsigned long long* g, unsigned char* sm,
                                         const BoxShared& S, GatherShared& gs, unsigned* stats)
        : A(a), grid(g), GS(gs), smem(sm) {
        if (!grid) return;   // nothing to gather (uniform across the CTA)
        const int npts = S.npts;
        const BoxGeom G = box_geom(S);
        const bool use = npts > 0 && G.vol <= kCap;
        if (use) load_gather_box<M>(A, grid, G, reinterpret_cast<float4*>(smem), reinterpret_cast<float*>(smem + 16 * kCap));
        if (threadIdx.x == 0) {
            gs.G = G;
            gs.use = use ? 1 : 0;
            if (stats && npts > 0) atomicAdd(stats + (use ? 2 : 3), 1u);
        }
        __syncthreads();
    }
    // Whether the box holds every cell the gather reads for corners C (those of
    // each axis: lo .. lo + cnt - 1).  A box computed from the points always
    // does; one stored by the previous step does only while the records are
    // the ones that step wrote, so a point that left it (records rewritten
    // through the device pointer, say) reads the grid directly instead.
    __device__ __forceinline__ bool holds(const BoxGeom& G, const Corners& C) const {
        bool ok = true;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax)
            ok = ok && (C.cnt[ax] <= 0 || (C.lo[ax] >= G.lo[ax] && C.lo[ax] + C.cnt[ax] <= G.lo[ax] + G.ext[ax]));
        return ok;
    }
    __device__ __forceinline__ f3 gather(f3 x, f3 v, float dt) const {
        const Corners C = corners_of<M>(A, x);
        if (GS.use && holds(GS.G, C)) {
            const float4* bf = reinterpret_cast<const float4*>(smem);
            const BoxGeom& G = GS.G;
            if constexpr (M::kExact) {
                const float* br = reinterpret_cast<const float*>(smem + 16 * kCap);
                return gather_point<M>(A, dt, x, v, C, [&](int a, int b, int c) {
                    const int li = G.offset(a, b, c);
                    const float4 q = bf[li];
                    return CellF{q.x, q.y, q.z, q.w, br[li]};
                });
            } else {
                return gather_point_fast(A, dt, v, C, G.offset(C.lo[0], C.lo[1], C.lo[2]), G.py, G.pz,
                                         [&](int i) { return bf[i]; });
            }
        }
        return gather_point_direct<M>(A, grid, dt, x, v);
    }
};

// ---- L2 prefetch ----------------------------------------------------------------
// Asks L2 to fetch `bytes` (a multiple of 16) at p (16-byte aligned); the
// thread does not wait.  L2 is the GPU's point of coherence, so a prefetch
// never returns stale data.
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Positions and velocities (adjacent in the record, 32 n bytes per strand) and
// rest lengths of strands [s0, s1), s0 a multiple of 8 (an item's first strand).  The rest buffer is
// allocated in 256-B units, so rounding its range up to 16 B stays inside.
__device__ __forceinline__ void prefetch_strands(const float4* strands, const float* rest, int n, int s0, int s1) {
    for (int s = s0 + (int)threadIdx.x; s < s1; s += kThreads)
        prefetch_l2(strands + (size_t)s * (3 * n), 32u * (unsigned)n);
    if (threadIdx.x == kThreads - 1 && s1 > s0) prefetch_l2(rest + s0, ((unsigned)(s1 - s0) * 4u + 15u) & ~15u);
}

// Strands [begin, end) of one asset in rounds of kWarps * (32/L) strands,
// handled in groups of U consecutive rounds that share one gather box and one
// splat box (fewer box loads, flushes and barriers than a box per round; a
// group's points stay below 4e9 / scale so its density partials stay exact):
//   1. (fused step) the group's current positions bound the box of
//      A.grid_prev, loaded once; each round then gathers the previous step's
//      loop 3 into its velocities;
//   2. each round runs loops 1-2 (strand_phase_a stores x', v, corr);
//   3. the group's new points, read back from this thread's own stores, are
//      splatted through one box.
// The round count is the same for every warp (the boxes synchronise the CTA).
template <int NFIX, int L, class M>
__device__ __forceinline__ void tile_a(const DevAsset& A, int begin, int end, unsigned char* smem, BoxShared& S,
                                       unsigned* stats) {
    constexpr int SPW = 32 / L;
    constexpr int K = PhaseA<NFIX, L>::K;
    const int n = NFIX > 0 ? NFIX : A.n_points;
    const int warp = threadIdx.x >> 5;
    const int g = (threadIdx.x & 31) / L;
    const int l = (threadIdx.x & 31) % L;
    const int per_round = kWarps * SPW;
    const int rounds = (end - begin + per_round - 1) / per_round;
    const float cap = 4.0e9f / (A.scale * (float)(per_round * n));   // rounds per group, density-exact
    const int Umax = max(1, min(kUnionRounds, (int)cap));
    const int U = A.group_rounds > 0 ? min(A.group_rounds, Umax) : Umax;
    // a warp's strands are spread over the round (neighbouring strands share cells)
    auto strand_of = [&](int r) { return begin + r * per_round + g * kWarps + warp; };
    const int first_round = begin / per_round;   // tiles start on round boundaries
    for (int r0 = 0; r0 < rounds; r0 += U) {
        const int r1 = min(rounds, r0 + U);
        int4* const gbox = A.group_box ? A.group_box + 2 * (first_round + r0) : nullptr;
        bool stored = false;   // the previous fused step left this group's box (uniform across the CTA)
        if (A.grid_prev && gbox && A.box_tag_read) {
            __shared__ int s_stored;
            if (threadIdx.x == 0) {
                const int4 lo = __ldcg(gbox), hi = __ldcg(gbox + 1);
                s_stored = (unsigned)lo.w == A.box_tag_read;
                if (s_stored) {
                    S.lo[0] = lo.x;
                    S.lo[1] = lo.y;
                    S.lo[2] = lo.z;
                    S.hi[0] = hi.x;
                    S.hi[1] = hi.y;
                    S.hi[2] = hi.z;
                    S.npts = hi.w;
                }
            }
            __syncthreads();
            stored = s_stored != 0;
            __syncthreads();   // s_stored is read by every thread before the next group writes it
        }
        if (A.grid_prev && !stored) {   // 1. the group's gather box (all of a pair of rounds' loads in flight)
            LaneBounds lb;
            for (int r = r0; r < r1; r += 2) {
                f3 xs[2][K];
                bool ok[2][K];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int strand = strand_of(r + h);
                    const bool valid = g < SPW && r + h < r1 && strand < end;
                    const float4* rec = A.strands + (size_t)(valid ? strand : 0) * (3 * n);
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        const int i = PhaseA<NFIX, L>::point(l, k);
                        ok[h][k] = valid && i >= 1 && i < n;
                        xs[h][k] = ok[h][k] ? xyz(ld_cg(rec + i)) : f3{0.f, 0.f, 0.f};
                    }
                }
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        if (ok[h][k]) lb.add(xs[h][k]);
            }
            lb.reduce<M>(A, S);
        }
        __shared__ GatherShared gs;
        const GatherBox<M> gb(A, A.grid_prev, smem, S, gs, stats);
        LaneBounds sb;
        for (int r = r0; r < r1; ++r) {   // 2. loops 1-2 per round
            const int strand = strand_of(r);
            const bool valid = g < SPW && strand < end;
            f3 x[K], v[K];
            const unsigned lmask = load_points<NFIX, L>(A, strand, valid, x, v);
            if (A.grid_prev)
                for_lane_points(x, v, lmask, [&](f3& p, f3& vel) { vel = gb.gather(p, vel, A.dt_prev); });
            f3 xo[K], vo[K];
            const unsigned mask = strand_phase_a<NFIX, L, M>(A, strand, valid, x, v, xo, vo);
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if (!((mask >> k) & 1u)) continue;
                sb.add(xo[k]);
                sb.add_v(vo[k]);
            }
        }
        if (A.grid_prev) __syncthreads();   // the gather box memory becomes the splat box
        if (A.grid_enabled) {   // 3. splat the group
            sb.reduce<M>(A, S);
            if (gbox && A.box_tag_write && threadIdx.x == 0) {   // the next fused step's gather box
                gbox[0] = make_int4(S.lo[0], S.lo[1], S.lo[2], (int)A.box_tag_write);
                gbox[1] = make_int4(S.hi[0], S.hi[1], S.hi[2], S.npts);
            }
            splat_points<L, M>(A, reinterpret_cast<int*>(smem), S, stats, [&](auto&& f) {
#pragma unroll 1
                for (int r = r0; r < r1; ++r) {
                    const int strand = strand_of(r);
                    const bool valid = g < SPW && strand < end;
                    const float4* rec = A.strands + (size_t)(valid ? strand : 0) * (3 * n);
                    // any order works for integer sums: lanes take blocks of K points, the
                    // block rotated by the strand's place in the warp, so the lanes of one
                    // instruction sit K points apart and the warp's strands at different
                    // heights (fewer lanes on one cell per shared atomic); the round's K
                    // points are loaded together, then splatted by a rolled loop
                    f3 ps[K], vs[K];
                    unsigned m = 0u;
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        const int i = ((l + 2 * g) % L) * K + k;
                        const bool ok = valid && i >= 1 && i < n;
                        ps[k] = ok ? xyz(rec[i]) : f3{0.f, 0.f, 0.f};
                        vs[k] = ok ? xyz(rec[n + i]) : f3{0.f, 0.f, 0.f};
                        if (ok) m |= 1u << k;
                    }
                    for_lane_points(ps, vs, m, [&](f3& p, f3& v) { f(p, v); });
                }
            });
        }
    }
}

// One thread per strand (lanes_per_strand = 1): strands [begin, end) of one
// asset in rounds of kThreads strands.  Each thread walks its strand from the
// root to the tip with a few registers of state, so any point count uses the
// same code and no lane repeats another's FTL chain:
//   1. (fused step) the cell box of the strand points' current positions is
//      loaded from A.grid_prev for the pending loop 3;
//   2. per point i = 1..n-1: pending gather + friction, collision force,
//      prediction, FTL from the moved parent, velocity, clamp, correction;
//      point i-1's DFTL term needs corr_i, so its velocity is stored one
//      point later (the last point gets none, compute.comp:213);
//   3. the round's new positions and velocities are read back (this thread's
//      own stores) and splatted through the shared box.
// Operation order per point is that of strand_phase_a, so exact math gives
// the same bits as every other path.
template <class M>
__device__ __forceinline__ void tile_a_stream(const DevAsset& A, int begin, int end, unsigned char* smem, BoxShared& S,
                                              unsigned* stats) {
    const int n = A.n_points;
    const float dt = A.dt;
    const float dt2 = M::mul(dt, dt);
    const bool moving = A.root_rest != nullptr;
    for (int r0 = begin; r0 < end; r0 += kThreads) {
        const int strand = r0 + (int)threadIdx.x;
        const bool valid = strand < end;
        const int np = valid ? n : 1;    // points this thread walks (none past the tile)
        float4* rec = A.strands + (size_t)(valid ? strand : 0) * (3 * n);

        // 1. the pending gather's box
        const bool pend_gather = A.grid_prev != nullptr;
        if (pend_gather) {
            LaneBounds lb;
            for (int i = 1; i < np; ++i) lb.add(xyz(rec[i]));
            lb.reduce<M>(A, S);
        }
        __shared__ GatherShared gs;
        const GatherBox<M> gb(A, A.grid_prev, smem, S, gs, stats);

        // 2. loops 1-2 along the strand
        f3 f0 = v_add<M>(f3{A.gravity[0], A.gravity[1], A.gravity[2]}, f3{A.wind[0], A.wind[1], A.wind[2]});
        if (A.strand_wind != nullptr && valid) f0 = v_add<M>(f0, xyz(A.strand_wind[strand]));
        const float r = valid ? A.rest[strand] : 0.f;
        f3 par = valid ? xyz(rec[0]) : f3{0.f, 0.f, 0.f};
        if (moving && valid) {
            par = head_point<M>(A.head, xyz(A.root_rest[strand]));
            st_f4(rec, par, 1.0f);
        }
        // optional copy of every new position (the root included) for the host
        float* const pxyz = A.pos_xyz != nullptr && valid ? A.pos_xyz + 3 * ((size_t)strand * n) : nullptr;
        if (pxyz) {
            pxyz[0] = par.x;
            pxyz[1] = par.y;
            pxyz[2] = par.z;
        }
        LaneBounds sb;
        f3 vprev = {0.f, 0.f, 0.f};
        for (int i = 1; i < np; ++i) {
            const f3 x = xyz(rec[i]);
            f3 v = xyz(rec[n + i]);
            if (pend_gather) v = gb.gather(x, v, A.dt_prev);
            const f3 force = collide_force<M>(A, x, f0);
            // predictedPos = currentPos + dt * currentVel + dt * dt * force   (compute.comp:187)
            const f3 p = v_axpy<M>(v_axpy<M>(x, dt, v), dt2, force);
            const f3 dir = v_normalize<M>(v_sub<M>(p, par));
            const f3 xn = v_axpy<M>(par, r, dir);
            const f3 newVel = v_div<M>(v_sub<M>(xn, x), dt);
            f3 vel = v_scale<M>(A.damping, newVel);
            if (v_len<M>(vel) > A.vmax) vel = v_scale<M>(A.vmax, v_normalize<M>(vel));
            const f3 cor = v_scale<M>(A.dftl, v_sub<M>(xn, p));
            st_f4(rec + i, xn, 1.0f);
            st_f4(rec + 2 * n + i, cor, 0.0f);
            if (pxyz) {
                pxyz[3 * i] = xn.x;
                pxyz[3 * i + 1] = xn.y;
                pxyz[3 * i + 2] = xn.z;
            }
            if (i >= 2) {   // point i-1: v -= corr_i / dt (compute.comp:213-215)
                vprev = v_sub<M>(vprev, v_div<M>(cor, dt));
                st_f4(rec + n + i - 1, vprev, 0.0f);
                sb.add_v(vprev);
            }
            vprev = vel;
            par = xn;
            sb.add(xn);
        }
        if (np >= 2) {
            st_f4(rec + n + np - 1, vprev, 0.0f);
            sb.add_v(vprev);
        }
        if (pend_gather) __syncthreads();   // the gather box memory is reused by the splat

        // 3. splat the round
        if (A.grid_enabled) {
            sb.reduce<M>(A, S);
            splat_points<1, M>(A, reinterpret_cast<int*>(smem), S, stats, [&](auto&& f) {
                for (int i = 1; i < np; ++i) f(xyz(rec[i]), xyz(rec[n + i]));
            });
        }
    }
}

// The generic point count, called out of line from the batch kernel: it is rare, and
// inlined its registers pushed the common paths into spills (k_batch<8, FastMath>: 692 B
// of spill stores with it and the phase-B tiles inline, 320 B without).
template <int L, class M>
__device__ __noinline__ void tile_a_generic(const DevAsset& A, int begin, int end, unsigned char* smem, BoxShared& S,
                                            unsigned* stats) {
    tile_a<0, L, M>(A, begin, end, smem, S, stats);
}

template <int L, class M>
__device__ __forceinline__ void tile_a_any(const DevAsset& A, int begin, int end, unsigned char* smem, BoxShared& S,
                                           unsigned* stats) {
    switch (A.n_points) {
        case 8: tile_a<8, L, M>(A, begin, end, smem, S, stats); break;
        case 16: tile_a<16, L, M>(A, begin, end, smem, S, stats); break;
        case 24: tile_a<24, L, M>(A, begin, end, smem, S, stats); break;
        case 32: tile_a<32, L, M>(A, begin, end, smem, S, stats); break;
        default: tile_a_generic<L, M>(A, begin, end, smem, S, stats); break;
    }
}

// Phase B (loop 3) for strands [s0, s1) of one asset, at most kTileB points.
// Thread t takes tile-local points t, t + kThreads, ...; 32-bit index math.
template <class M>
__device__ __forceinline__ void tile_b(const DevAsset& A, int s0, int s1, unsigned char* smem, BoxShared& S,
                                       unsigned* stats) {
    const int n = A.n_points;
    const int npt = (s1 - s0) * n;
    float4* const base = A.strands + (size_t)s0 * (3 * n);
    const FastDiv dn((unsigned)n);
    f3 x[kPtsB];
    int off[kPtsB];   // record offset (float4 units) of the point's curvePoints slot
    unsigned m = 0u;
    LaneBounds lb;
#pragma unroll
    for (int j = 0; j < kPtsB; ++j) {
        const int q = threadIdx.x + j * kThreads;
        x[j] = f3{0.f, 0.f, 0.f};
        off[j] = 0;
        if (q >= npt) continue;
        const int ls = (int)dn.div((unsigned)q);
        const int i = q - ls * n;
        if (i == 0) continue;
        off[j] = ls * (3 * n) + i;
        x[j] = xyz(ld_cg(base + off[j]));
        m |= 1u << j;
        lb.add(x[j]);
    }
    lb.reduce<M>(A, S);
    __shared__ GatherShared gs;
    const GatherBox<M> gb(A, A.grid, smem, S, gs, stats);
#pragma unroll
    for (int j = 0; j < kPtsB; ++j) {
        if (!((m >> j) & 1u)) continue;
        float4* vp = base + off[j] + n;
        st_f4(vp, gb.gather(x[j], xyz(ld_cg(vp)), A.dt), 0.0f);
    }
    __syncthreads();  // every read of S and of the box is done before the next tile resets them
}

__device__ __forceinline__ void write_draw(const DevAsset& A) {
    if (A.draw) {
        A.draw->vertex_count = (uint32_t)A.n_strands;  // compute.comp:302, one per strand
        A.draw->instance_count = 1u;
        A.draw->first_vertex = 0u;
        A.draw->first_instance = 0u;
    }
}

// ---- plain path -------------------------------------------------------------

template <int NFIX, int L, class M>
__global__ void __launch_bounds__(kThreads, kMinCtasPerSm) k_plain_a(const __grid_constant__ DevAsset A) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ BoxShared S;
    constexpr int SPW = 32 / L;
    const int begin = blockIdx.x * kWarps * SPW;
    const int end = min(begin + kWarps * SPW, A.n_strands);
    tile_a<NFIX, L, M>(A, begin, end, dsm, S, nullptr);
    if (!A.grid_enabled && blockIdx.x == 0 && threadIdx.x == 0) write_draw(A);
}

template <class M>
__global__ void __launch_bounds__(kThreads, kMinCtasPerSm) k_plain_b(const __grid_constant__ DevAsset A) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ BoxShared S;
    const int per_tile = max(1, kTileB / A.n_points);
    for (int s0 = blockIdx.x * per_tile; s0 < A.n_strands; s0 += gridDim.x * per_tile)
        tile_b<M>(A, s0, min(A.n_strands, s0 + per_tile), dsm, S, nullptr);
    if (blockIdx.x == 0 && threadIdx.x == 0) write_draw(A);
}

// ---- batched persistent path -----------------------------------------------
// Phase-B tiles, called out of line from the batch kernel for the same reason (only the
// full-step and finishing modes queue them).
template <class M>
__device__ __noinline__ void tile_b_out(const DevAsset& A, int s0, int s1, unsigned char* smem, BoxShared& S,
                                        unsigned* stats) {
    tile_b<M>(A, s0, s1, smem, S, stats);
}

template <int L, class M>
__global__ void __launch_bounds__(kThreads, kMinCtasPerSm) k_batch(const __grid_constant__ BatchDev B) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ BoxShared S;
    __shared__ int s_item, s_next;
    __shared__ int s_asset;
    // The current item's asset, copied once into shared memory: reads of its
    // fields then cannot alias the global stores of the step.
    __shared__ __align__(16) DevAsset A;
    // Each CTA holds the item after its current one (taken from the queue in
    // order, so every wait is still on an earlier item) and, when it is a
    // phase-A item and items are large, asks L2 for its strands while the
    // current one runs (with items of one or two rounds the prefetch only
    // duplicates the demand loads: a 100k-strand head stepped 2 % slower).
    if (threadIdx.x == 0) {
        s_asset = -1;
        s_next = (int)atomicAdd(B.head, 1u);
    }
    for (;;) {
        __syncthreads();   // the previous item is done and s_next is visible
        if (threadIdx.x == 0) {
            s_item = s_next;
            s_next = s_item < B.n_items ? (int)atomicAdd(B.head, 1u) : B.n_items;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= B.n_items) break;
        if (B.prefetch && s_next < B.n_items) {
            const WorkItem wn = B.items[s_next];
            if (wn.kind == ITEM_A) {
                const DevAsset* N = B.assets + wn.asset;
                prefetch_strands(N->strands, N->rest, N->n_points, wn.begin, wn.end);
            }
        }
        const WorkItem w = B.items[it];
        if (w.asset != s_asset) {
            constexpr int words = (int)(sizeof(DevAsset) / 4);
            const int* src = reinterpret_cast<const int*>(B.assets + w.asset);
            int* dst = reinterpret_cast<int*>(&A);
            for (int q = threadIdx.x; q < words; q += kThreads) dst[q] = src[q];
            __syncthreads();
            if (threadIdx.x == 0) s_asset = w.asset;
        }
        if (w.kind != ITEM_B && A.wait_entry >= 0) {   // a later step of the same asset
            if (threadIdx.x == 0) {
                const unsigned need = B.need_a[A.wait_entry];
                uint32_t spins = 0;
                while (ld_acquire_gpu(B.done_a + A.wait_entry) < need) {
                    if (++spins > B.spin_limit) {
                        atomicExch(B.error, RVH_ERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(256);
                }
            }
            __syncthreads();
        }
        if (w.kind == ITEM_A) {
            if constexpr (L == 1) tile_a_stream<M>(A, w.begin, w.end, dsm, S, B.stats);
            else tile_a_any<L, M>(A, w.begin, w.end, dsm, S, B.stats);
            if (!A.grid_enabled && w.begin == 0 && threadIdx.x == 0) write_draw(A);
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                atomicAdd(B.done_a + w.asset, 1u);
            }
        } else if (w.kind == ITEM_B) {
            if (threadIdx.x == 0) {
                const unsigned need = B.need_a[w.asset];
                uint32_t spins = 0;
                while (ld_acquire_gpu(B.done_a + w.asset) < need) {
                    if (++spins > B.spin_limit) {
                        atomicExch(B.error, RVH_ERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(256);
                }
            }
            __syncthreads();
            tile_b_out<M>(A, w.begin, w.end, dsm, S, B.stats);
            if (w.begin == 0 && threadIdx.x == 0) write_draw(A);
        } else {
            uint4* g = reinterpret_cast<uint4*>(A.grid_next);
            for (int c = w.begin + threadIdx.x; c < w.end; c += kThreads) g[c] = make_uint4(0u, 0u, 0u, 0u);
            __syncthreads();
            if (B.count_clears && threadIdx.x == 0) {   // a later step of this asset splats here
                __threadfence();
                atomicAdd(B.done_a + w.asset, 1u);
            }
        }
    }
}

}  // namespace rvh
