// rvh_health.cu — failure detection for a running simulation.
//
// The reference has none (its state is only ever drawn).  rvh_asset_health
// scans an asset's Strand records on the device and reports what a blown-up
// or corrupted simulation shows first: non-finite positions or velocities, the
// largest speed (clamped to vmax before the DFTL correction and the friction
// blend, compute.comp:198-215, so a healthy state can exceed vmax), and the
// largest inextensibility error |segment - rest| / (rest * (n - 1)) that FTL
// keeps near rounding (compute.comp:191-192).  One thread per strand; the
// maxima are atomic maxima of the float bits (non-negative values order like
// their bits), the worst strand packed below the error.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "rvh_internal.hpp"

namespace rvh {
namespace {

constexpr int kHealthThreads = 256;

struct HealthDev {
    unsigned long long nonfinite;
    unsigned max_speed_bits;
    unsigned pad;
    unsigned long long worst;   // (error bits << 32) | strand
};

__device__ __forceinline__ bool finite3(float4 q) { return isfinite(q.x) && isfinite(q.y) && isfinite(q.z); }

__global__ void __launch_bounds__(kHealthThreads) k_health(const float4* __restrict__ strands,
                                                           const float* __restrict__ rest, int n_strands, int n,
                                                           HealthDev* __restrict__ out) {
    unsigned long long bad = 0;
    float vmax = 0.f;
    unsigned long long worst = 0;
    for (int s = blockIdx.x * kHealthThreads + threadIdx.x; s < n_strands; s += gridDim.x * kHealthThreads) {
        const float4* rec = strands + (size_t)s * (3 * n);
        const float r = rest[s];
        const float L = r * (float)(n - 1);
        float4 prev = __ldg(rec);
        bad += !finite3(prev);
        float err = 0.f;
        for (int i = 0; i < n; ++i) {
            const float4 x = i == 0 ? prev : __ldg(rec + i);
            const float4 v = __ldg(rec + n + i);
            if (i > 0) bad += !finite3(x);
            if (!finite3(v)) {
                ++bad;
            } else {
                vmax = fmaxf(vmax, sqrtf(v.x * v.x + v.y * v.y + v.z * v.z));
            }
            if (i > 0 && finite3(x) && finite3(prev) && L > 0.f) {
                const float dx = x.x - prev.x, dy = x.y - prev.y, dz = x.z - prev.z;
                const float e = fabsf(sqrtf(dx * dx + dy * dy + dz * dz) - r) / L;
                err = fmaxf(err, e);
            }
            prev = x;
        }
        const unsigned long long key = ((unsigned long long)__float_as_uint(err) << 32) | (unsigned)s;
        worst = key > worst ? key : worst;
    }
    // warp reductions, then one atomic per warp
    for (int off = 16; off > 0; off >>= 1) {
        bad += __shfl_down_sync(0xffffffffu, bad, off);
        vmax = fmaxf(vmax, __shfl_down_sync(0xffffffffu, vmax, off));
        const unsigned long long w = __shfl_down_sync(0xffffffffu, worst, off);
        worst = w > worst ? w : worst;
    }
    if ((threadIdx.x & 31) == 0) {
        if (bad) atomicAdd(&out->nonfinite, bad);
        atomicMax(&out->max_speed_bits, __float_as_uint(vmax));
        atomicMax(&out->worst, worst);
    }
}

}  // namespace
}  // namespace rvh

using namespace rvh;

extern "C" {

rvh_status rvh_asset_health(rvh_asset* a, rvh_health* out) {
    TraceRange trace("rvh_asset_health");
    if (!a || !out) return fail(RVH_ERR_INVALID_ARG, "asset_health: NULL argument");
    *out = rvh_health{};
    out->worst_strand = -1;
    if (a->n_strands == 0) return RVH_OK;
    RVH_DEVICE(a->ctx->device);
    rvh_status st = finish_pending(a, a->ctx->stream);
    if (st != RVH_OK) return st;
    DevBuf buf;
    if ((st = a->ctx->alloc(buf, sizeof(HealthDev))) != RVH_OK) return st;
    cudaStream_t s = a->ctx->stream;
    cudaError_t e = cudaMemsetAsync(buf.ptr, 0, sizeof(HealthDev), s);
    if (e == cudaSuccess) {
        const int blocks = (int)std::min<long long>(((long long)a->n_strands + kHealthThreads - 1) / kHealthThreads,
                                                    (long long)a->ctx->sm_count * 8);
        k_health<<<blocks, kHealthThreads, 0, s>>>(static_cast<const float4*>(a->strands.ptr),
                                                   static_cast<const float*>(a->rest.ptr), a->n_strands, a->n_points,
                                                   static_cast<HealthDev*>(buf.ptr));
        e = cudaGetLastError();
    }
    HealthDev h{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, buf.ptr, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    a->ctx->free(buf);
    if (e != cudaSuccess) return cuda_fail(e, "asset_health");
    out->nonfinite = h.nonfinite;
    std::memcpy(&out->max_speed, &h.max_speed_bits, 4);
    const unsigned eb = (unsigned)(h.worst >> 32);
    std::memcpy(&out->max_length_error, &eb, 4);
    out->worst_strand = (int32_t)(h.worst & 0xffffffffu);
    return RVH_OK;
}

}  // extern "C"
