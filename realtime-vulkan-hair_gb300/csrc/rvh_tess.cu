// rvh_tess.cu — strand tessellation into render-ready polylines.
//
// The reference tessellates each guide strand on the GPU's fixed-function
// tessellator: hair.tesc:19-20 asks for 12 isolines of 42 segments, and
// hair.tese emits, per isoline vertex, a point on a cubic Bezier through the
// strand's points offset by a clump width along a per-isoline direction
// (single-strand clumping, hair.tese:153-330; the multi-strand blend it also
// computes is overwritten at :311).  There is no graphics pipeline here, so
// this kernel writes the same vertices to a device buffer a renderer (or a
// file) consumes:
//
//   vertex (strand s, isoline j, vertex k) = float4 {position, strand width}
//   u = j / n_lines, v = k / n_segments (gl_TessCoord.y, .x)
//   segment sf = floor(v (n-1)), t = v (n-1) - sf; control points from the
//   four surrounding points, end neighbours mirrored (hair.tese:45-66);
//   de Casteljau with mix(a, b, t) = a + t (b - a) (:69-77)
//   pos = c + width(j, k) * dir(j) * sd(profile(s, j), k)           (:237-308)
//   width = mix(rootWidth, tipWidth, v)                              (:324-326)
//   optional per-segment frames {tangent, Frisvad b1, b2}            (:289-297)
//
// A CTA of 256 threads takes 16 strands at a time: their points and Bezier
// control points in shared memory, their (strand, isoline) sd profiles, then
// one thread per (strand, vertex column): the curve point is evaluated once and
// offset for every isoline, with coalesced float4 stores.
//
// Everything that depends only on (isoline, vertex) — the clump width, the
// direction, the five sd profiles of v, the strand width — is a table the
// host computes once per descriptor with the C library's float functions.
// The per-strand hash random(st) = fract(sin(dot(st, (12.9898, 78.233))) *
// 43758.5453123) (:29-31) picks the sd profile; its sin is evaluated in double
// and rounded once (a correctly rounded float sin), so every host and the GPU
// agree.  The profiles are cached per strand with the root bits they came from
// and recomputed only for strands whose root moved.  All float arithmetic is separately rounded, in the shader's order.
// Two definitions where the shader is undefined: at v = 1 it reads point n
// (out of bounds) — here the curve ends at the tip (last segment, t = 1); and
// n is the asset's point count (the shader fixes 10).
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "rvh_internal.hpp"
#include "rvh_kernels.cuh"

namespace rvh {
namespace {

constexpr int kTessThreads = 256;
constexpr int kTessGroup = 16;   // strands per CTA iteration
constexpr int kMaxLines = 64;
constexpr int kMaxSegments = 256;

using EM = ExactMath;

__device__ __forceinline__ float tess_random_dev(float x, float y) {
    const float d = EM::add(EM::mul(x, 12.9898f), EM::mul(y, 78.233f));
    const float s = (float)sin((double)d);
    const float m = EM::mul(s, 43758.5453123f);
    return EM::sub(m, floorf(m));
}

__device__ __forceinline__ f3 e_mix(f3 a, f3 b, float t) { return v_add<EM>(a, v_scale<EM>(t, v_sub<EM>(b, a))); }

// Frisvad's orthonormal basis of unit n (hair.tese:140-151)
__device__ __forceinline__ void frisvad_dev(f3 n, f3& b1, f3& b2) {
    if (n.z < -0.9999999f) {
        b1 = f3{0.0f, -1.0f, 0.0f};
        b2 = f3{-1.0f, 0.0f, 0.0f};
        return;
    }
    const float a = EM::div(1.0f, EM::add(1.0f, n.z));
    const float b = EM::mul(EM::mul(-n.x, n.y), a);
    b1 = v_normalize<EM>(f3{EM::sub(1.0f, EM::mul(EM::mul(n.x, n.x), a)), b, -n.x});
    b2 = v_normalize<EM>(f3{b, EM::sub(1.0f, EM::mul(EM::mul(n.y, n.y), a)), -n.y});
}

// Device tables: u[L], v[S+1], width[L][S+1], dir[L] (xyz), sd[6][S+1], strand width[S+1]
struct TessTablesDev {
    const float* u;
    const float* v;
    const float* width;
    const float* dir;
    const float* sd;
    const float* sw;
};

// Profile cache: the sd profile of (strand, isoline) depends only on the
// strand's root and the isoline, and roots move only with a head motion (or a
// write of the records).  Each strand keeps the root bits its cached profiles
// were computed from; a strand whose root bits are unchanged reuses them, any
// other strand recomputes (the same function, so the bits never differ).
struct TessCacheDev {
    uint4* roots;            // per strand: root x, y, z bits (w unused); all ones before the first call
    unsigned char* prof;     // per strand: n_lines profiles
};

struct TessArgs {
    const float4* strands;
    int n_strands, n_points, n_lines, n_segments;
    TessTablesDev T;
    TessCacheDev C;          // roots == nullptr: no cache
    float4* out;
    float4* frames;
};

__device__ __forceinline__ int tess_profile(float u, f3 root) {
    const float choice = EM::mul(tess_random_dev(u, root.x), tess_random_dev(root.y, root.z));
    int p = 0;
    if (choice > 0.5f) p = choice > 0.9f ? 1 : choice > 0.8f ? 2 : choice > 0.7f ? 3 : choice > 0.6f ? 4 : 5;
    return p;
}

__global__ void __launch_bounds__(kTessThreads) k_tessellate(const __grid_constant__ TessArgs A) {
    __shared__ f3 pts[kTessGroup][RVH_MAX_POINTS];
    __shared__ f3 cb1[kTessGroup][RVH_MAX_POINTS], cb2[kTessGroup][RVH_MAX_POINTS];
    __shared__ int prof[kTessGroup][kMaxLines];
    const int n = A.n_points, L = A.n_lines, S1 = A.n_segments + 1;
    const int per_strand = L * S1;
    const FastDiv dS1((unsigned)S1), dL((unsigned)L);
    // the group's points: slot t = threadIdx.x + m * kTessThreads holds point t % 32
    // of strand t / 32; a thread's slots of the next group are loaded into
    // registers while the current group's vertices are written
    constexpr int kSlots = kTessGroup * RVH_MAX_POINTS / kTessThreads;
    static_assert(kSlots * kTessThreads == kTessGroup * RVH_MAX_POINTS, "slots per thread");
    const int stride = gridDim.x * kTessGroup;
    float4 next[kSlots];
    auto load_group = [&](int s) {
        const int ngs = min(kTessGroup, A.n_strands - s);
#pragma unroll
        for (int m = 0; m < kSlots; ++m) {
            const int t = threadIdx.x + m * kTessThreads, g = t / RVH_MAX_POINTS, i = t % RVH_MAX_POINTS;
            if (s < A.n_strands && g < ngs && i < n) next[m] = A.strands[(size_t)(s + g) * (3 * n) + i];
        }
    };
    load_group(blockIdx.x * kTessGroup);
    for (int s0 = blockIdx.x * kTessGroup; s0 < A.n_strands; s0 += stride) {
        const int ng = min(kTessGroup, A.n_strands - s0);   // strands of this group
#pragma unroll
        for (int m = 0; m < kSlots; ++m) {
            const int t = threadIdx.x + m * kTessThreads, g = t / RVH_MAX_POINTS, i = t % RVH_MAX_POINTS;
            if (g < ng && i < n) pts[g][i] = xyz(next[m]);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < kTessGroup * RVH_MAX_POINTS; t += kTessThreads) {
            // control points and frame of segment sf (hair.tese:45-66)
            const int g = t / RVH_MAX_POINTS, sf = t % RVH_MAX_POINTS;
            if (g < ng && sf + 1 < n) {
                const f3 p1 = pts[g][sf], p2 = pts[g][sf + 1];
                const f3 p0 = sf == 0 ? v_add<EM>(p1, v_sub<EM>(p1, p2)) : pts[g][sf - 1];
                const f3 p3 = sf + 1 == n - 1 ? v_add<EM>(p2, v_sub<EM>(p2, p1)) : pts[g][sf + 2];
                const float third = 1.0f / 3.0f;
                cb1[g][sf] = v_add<EM>(p1, v_scale<EM>(third, v_div<EM>(v_sub<EM>(p2, p0), 2.0f)));
                cb2[g][sf] = v_sub<EM>(p2, v_scale<EM>(third, v_div<EM>(v_sub<EM>(p3, p1), 2.0f)));
                if (A.frames) {
                    const f3 tg = v_normalize<EM>(v_sub<EM>(p2, p1));
                    f3 b1, b2;
                    frisvad_dev(tg, b1, b2);
                    float4* fr = A.frames + ((size_t)(s0 + g) * (n - 1) + sf) * 3;
                    fr[0] = make_float4(tg.x, tg.y, tg.z, 0.f);
                    fr[1] = make_float4(b1.x, b1.y, b1.z, 0.f);
                    fr[2] = make_float4(b2.x, b2.y, b2.z, 0.f);
                }
            }
        }
        // sd profile of (strand, isoline): randomChoice (hair.tese:253-283), from
        // the cache when the strand's root bits are those it was computed from
        for (int q = threadIdx.x; q < ng * L; q += kTessThreads) {
            const int g = (int)dL.div((unsigned)q), j = q - g * L;
            const f3 root = pts[g][0];
            int p;
            if (A.C.roots != nullptr) {
                const uint4 cr = A.C.roots[s0 + g];
                unsigned char* cp = A.C.prof + (size_t)(s0 + g) * L + j;
                if (cr.x == __float_as_uint(root.x) && cr.y == __float_as_uint(root.y) &&
                    cr.z == __float_as_uint(root.z)) {
                    p = *cp;
                } else {
                    p = tess_profile(A.T.u[j], root);
                    *cp = (unsigned char)p;
                }
            } else {
                p = tess_profile(A.T.u[j], root);
            }
            prof[g][j] = p;
        }
        __syncthreads();
        if (A.C.roots != nullptr && threadIdx.x < ng) {   // every comparison above is done
            const f3 root = pts[threadIdx.x][0];
            A.C.roots[s0 + threadIdx.x] =
                make_uint4(__float_as_uint(root.x), __float_as_uint(root.y), __float_as_uint(root.z), 0u);
        }
        load_group(s0 + stride);   // in flight during the stores below
        // the curve point c(v) of (strand, vertex k) is the same for every isoline:
        // one thread per (strand, k) evaluates it once and writes the strand's
        // n_lines vertices of column k (consecutive threads: consecutive k of one
        // isoline row, coalesced)
        float4* out = A.out + (size_t)s0 * per_strand;
        for (int q = threadIdx.x; q < ng * S1; q += kTessThreads) {
            const int g = (int)dS1.div((unsigned)q), k = q - g * S1;
            const float v = __ldg(A.T.v + k);
            const float x = EM::mul(v, (float)(n - 1));
            int sf = (int)floorf(x);
            sf = min(sf, n - 2);
            const float t = EM::sub(x, (float)sf);
            const f3 b0 = pts[g][sf], b1 = cb1[g][sf], b2 = cb2[g][sf], b3 = pts[g][sf + 1];
            const f3 b01 = e_mix(b0, b1, t), b11 = e_mix(b1, b2, t), b21 = e_mix(b2, b3, t);
            const f3 b02 = e_mix(b01, b11, t), b12 = e_mix(b11, b21, t);
            const f3 c = e_mix(b02, b12, t);
            const float sw = __ldg(A.T.sw + k);
            float4* col = out + (size_t)g * per_strand + k;
            for (int j = 0; j < L; ++j) {
                const float sd = __ldg(A.T.sd + prof[g][j] * S1 + k);
                const f3 dir = v_scale<EM>(sd, f3{__ldg(A.T.dir + 3 * j), __ldg(A.T.dir + 3 * j + 1),
                                                  __ldg(A.T.dir + 3 * j + 2)});
                const f3 pos = v_add<EM>(c, v_scale<EM>(__ldg(A.T.width + j * S1 + k), dir));
                col[(size_t)j * S1] = make_float4(pos.x, pos.y, pos.z, sw);
            }
        }
        __syncthreads();   // pts, cb1/cb2 and prof are rewritten for the next group
    }
}

// ---- host tables ---------------------------------------------------------------

float h_fract(float x) { return x - std::floor(x); }
float h_mix(float a, float b, float t) { return a + t * (b - a); }
float h_random(float x, float y) {
    const float d = x * 12.9898f + y * 78.233f;
    return h_fract((float)std::sin((double)d) * 43758.5453123f);
}

// Packs the tables in the order of TessTablesDev: u, v, width, dir, sd, sw.
std::vector<float> host_tables(const rvh_tess_desc& d, size_t off[6]) {
    const int L = d.n_lines, S = d.n_segments;
    std::vector<float> u(L), v(S + 1), width, dir, sd, sw;
    for (int j = 0; j < L; ++j) u[j] = (float)j / (float)L;
    for (int k = 0; k <= S; ++k) v[k] = (float)k / (float)S;
    const float PI = 3.141592653f;
    for (int j = 0; j < L; ++j) {
        const float rand2 = std::fabs(h_random(u[j], u[j] * u[j]));
        for (int k = 0; k <= S; ++k)
            width.push_back(d.clump_radius * h_mix(h_mix(0.05f, 0.3f, v[k]), h_mix(0.3f, 0.1f, v[k]), v[k]) *
                            (rand2 + 0.5f));
        const float uRad = 2.f * PI * u[j];
        const float c = std::cos(uRad), s = std::sin(uRad);
        const float inv = 1.0f / std::sqrt((c * c + 0.f * 0.f) + s * s);
        dir.push_back(c * inv);
        dir.push_back(0.f * inv);
        dir.push_back(s * inv);
    }
    const float den = 2.0f * std::pow(0.2f, 2.0f);
    for (int p = 0; p < 6; ++p)
        for (int k = 0; k <= S; ++k) {
            float x = 1.0f;
            switch (p) {
                case 1: x = 1.8f * std::exp(-std::pow(v[k] - 0.25f, 2.0f) / den); break;
                case 2: x = 4.5f * std::pow(v[k], 10.0f); break;
                case 3: x = 2.5f * std::exp(-std::pow(v[k] - 0.7f, 2.0f) / den); break;
                case 4: x = 4.f * std::pow(v[k], 1.3f); break;
                case 5: x = 1.8f * std::exp(-std::pow(v[k] - 0.8f, 2.0f) / den); break;
                default: break;
            }
            if (v[k] == 0.0f) x = 1.0f;
            sd.push_back(x);
        }
    for (int k = 0; k <= S; ++k) sw.push_back(h_mix(d.root_width, d.tip_width, v[k]));
    std::vector<float> all;
    const std::vector<float>* parts[6] = {&u, &v, &width, &dir, &sd, &sw};
    for (int i = 0; i < 6; ++i) {
        off[i] = all.size();
        all.insert(all.end(), parts[i]->begin(), parts[i]->end());
        while (all.size() % 4) all.push_back(0.f);   // 16-byte aligned parts
    }
    return all;
}

bool same_desc(const rvh_tess_desc& a, const rvh_tess_desc& b) { return std::memcmp(&a, &b, sizeof a) == 0; }

}  // namespace
}  // namespace rvh

using namespace rvh;

extern "C" {

rvh_status rvh_tess_desc_reference(rvh_tess_desc* d) {
    if (!d) return fail(RVH_ERR_INVALID_ARG, "tess_desc_reference: NULL");
    std::memset(d, 0, sizeof(*d));
    d->n_lines = 12;        // hair.tesc:19
    d->n_segments = 42;     // hair.tesc:20
    d->clump_radius = 0.5f; // hair.tese:239
    d->root_width = 0.02f;  // hair.tese:324
    d->tip_width = 0.01f;   // hair.tese:325
    return RVH_OK;
}

rvh_status rvh_asset_tessellate(rvh_asset* a, const rvh_tess_desc* d, void* vertices, void* frames, void* stream) {
    TraceRange trace("rvh_asset_tessellate");
    if (!a || !d) return fail(RVH_ERR_INVALID_ARG, "asset_tessellate: NULL argument");
    if (d->n_lines < 1 || d->n_lines > kMaxLines || d->n_segments < 1 || d->n_segments > kMaxSegments)
        return fail(RVH_ERR_INVALID_ARG, "asset_tessellate: n_lines must be in [1, 64], n_segments in [1, 256]");
    if (!std::isfinite(d->clump_radius) || !std::isfinite(d->root_width) || !std::isfinite(d->tip_width))
        return fail(RVH_ERR_INVALID_ARG, "asset_tessellate: non-finite constants");
    if (a->n_strands > 0 && !vertices) return fail(RVH_ERR_INVALID_ARG, "asset_tessellate: vertices is NULL");
    if (reinterpret_cast<uintptr_t>(vertices) % 16 || reinterpret_cast<uintptr_t>(frames) % 16)
        return fail(RVH_ERR_INVALID_ARG, "asset_tessellate: buffers must be 16-byte aligned");
    if (a->n_strands == 0) return RVH_OK;
    RVH_CUDA(cudaSetDevice(a->ctx->device));
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : a->ctx->stream;
    // pending friction only changes velocities; positions are final, so no finish is needed
    if (!a->tess_tables.ptr || !same_desc(a->tess_desc, *d)) {
        size_t off[6];
        const std::vector<float> tab = host_tables(*d, off);
        a->ctx->free(a->tess_tables);
        rvh_status st = a->ctx->alloc(a->tess_tables, tab.size() * sizeof(float));
        if (st != RVH_OK) return st;
        RVH_CUDA(cudaStreamSynchronize(s));
        RVH_CUDA(cudaMemcpy(a->tess_tables.ptr, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
        a->tess_desc = *d;
        std::memcpy(a->tess_off, off, sizeof off);
        // a new descriptor: the profile cache starts empty (roots all ones, profiles 0);
        // without room for it every call recomputes the profiles
        a->ctx->free(a->tess_cache);
        const size_t rb = size_t(a->n_strands) * 16u, pb = size_t(a->n_strands) * size_t(d->n_lines);
        const std::string keep = last_error_cstr();   // a cache that does not fit is not an error
        if (a->ctx->alloc(a->tess_cache, rb + ((pb + 15u) & ~size_t(15))) == RVH_OK) {
            RVH_CUDA(cudaMemsetAsync(a->tess_cache.ptr, 0xff, rb, s));
            RVH_CUDA(cudaMemsetAsync(static_cast<unsigned char*>(a->tess_cache.ptr) + rb, 0, pb, s));
        } else {
            set_error(keep);
        }
    }
    const float* base = static_cast<const float*>(a->tess_tables.ptr);
    TessArgs A{};
    A.strands = static_cast<const float4*>(a->strands.ptr);
    A.n_strands = a->n_strands;
    A.n_points = a->n_points;
    A.n_lines = d->n_lines;
    A.n_segments = d->n_segments;
    A.T = TessTablesDev{base + a->tess_off[0], base + a->tess_off[1], base + a->tess_off[2],
                        base + a->tess_off[3], base + a->tess_off[4], base + a->tess_off[5]};
    if (a->tess_cache.ptr) {
        A.C.roots = static_cast<uint4*>(a->tess_cache.ptr);
        A.C.prof = static_cast<unsigned char*>(a->tess_cache.ptr) + size_t(a->n_strands) * 16u;
    }
    A.out = static_cast<float4*>(vertices);
    A.frames = static_cast<float4*>(frames);
    // one wave of resident CTAs, each walking its groups
    static int per_sm = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tessellate, kTessThreads, 0) != cudaSuccess)
            per_sm = 0;
    });
    const long long groups = (a->n_strands + kTessGroup - 1) / kTessGroup;
    const int blocks = (int)std::min<long long>(groups, (long long)a->ctx->sm_count * std::max(1, per_sm));
    void* args[] = {&A};
    RVH_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(&k_tessellate), dim3(blocks), dim3(kTessThreads), args, 0, s));
    return RVH_OK;
}

}  // extern "C"
