// rvh_noalloc.cu — the plain hair step for callers that cannot let the
// library allocate device memory.
//
// Some callers own every device buffer themselves and cannot have a plugin
// allocate: a real-time frame loop where a cudaMalloc (which may synchronise
// the device) would stall the frame, or a host application whose own
// allocator hands out all GPU memory and forbids allocations by the code it
// loads.  rvh_step_noalloc takes the caller's buffers (Strand records, rest
// lengths, optional per-strand wind and draw record) and keeps its only
// scratch, the hair-hair grid, in the file-scope array below.  It calls no
// cudaMalloc, cudaFree or other allocating routine.
//
// The array holds RVH_NOALLOC_MAX_GRID_CELLS cells (4 x int64 each, 8 MiB);
// every GPU that loads the library keeps it until the process exits.  All
// calls on one device share that device's copy: each call clears the cells it
// uses before splatting, and calls whose work overlaps on the GPU (for
// example on two streams) race on it, so a caller must order them.  The first
// call on a device (and the first after that device's context was torn down,
// e.g. by cudaDeviceReset) looks up the array's device address; make that
// first call before any stream capture.
#include <cuda.h>

#include <mutex>

#include "rvh_internal.hpp"
#include "rvh_registry.h"

namespace rvh {
namespace {

static __device__ __align__(256) unsigned long long g_noalloc_grid[size_t(RVH_NOALLOC_MAX_GRID_CELLS) * 4];

// Writes the draw record of an empty step (no strands): vertexCount 0.
__global__ void k_noalloc_empty_draw(rvh_draw_indirect* d) {
    d->vertex_count = 0u;
    d->instance_count = 1u;
    d->first_vertex = 0u;
    d->first_instance = 0u;
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct ScratchAddr {
    void* ptr = nullptr;
    unsigned long long ctx_id = 0;   // the context the address belongs to (0: unknown)
};
ScratchAddr g_addr[kMaxDevices];

// Unique id of the calling thread's current context, or 0 when there is none
// or the driver cannot say (then the address is looked up on every call).
// cuCtxGetId ids are never reused within a process, so a context that was
// torn down and created again gets a new one.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    });
    if (!get_current || !get_id) return 0;
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on the current device `dev`, looked up
// with that device current on its first call and again whenever the current
// context is not the one the cached address was taken in.
rvh_status scratch_address(int dev, void** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(RVH_ERR_UNSUPPORTED, "step_noalloc: device ordinal too large");
    std::lock_guard<std::mutex> g(g_mu);
    ScratchAddr& a = g_addr[dev];
    const unsigned long long id = current_context_id();
    if (!a.ptr || id == 0 || id != a.ctx_id) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_grid);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc grid)");
        a.ptr = p;
        a.ctx_id = current_context_id();   // the lookup has made the device's context current
    }
    *out = a.ptr;
    return RVH_OK;
}

}  // namespace
}  // namespace rvh

using namespace rvh;

extern "C" {

rvh_status rvh_step_noalloc(const rvh_noalloc_step_desc* d, const rvh_frame* frame, void* stream) {
    if (!d || !frame || !d->params) return fail(RVH_ERR_INVALID_ARG, "step_noalloc: NULL argument");
    if (d->n_strands < 0 || d->n_points < RVH_MIN_POINTS || d->n_points > RVH_MAX_POINTS)
        return fail(RVH_ERR_INVALID_ARG, "step_noalloc: n_points must be in [2, 32] and n_strands >= 0");
    if (d->n_strands > 0 && (!d->strands || !d->rest_lengths))
        return fail(RVH_ERR_INVALID_ARG, "step_noalloc: strands and rest_lengths are required");
    if (reinterpret_cast<uintptr_t>(d->strands) % 16 != 0 || reinterpret_cast<uintptr_t>(d->strand_wind) % 16 != 0)
        return fail(RVH_ERR_INVALID_ARG, "step_noalloc: strands and strand_wind must be 16-byte aligned");
    if (d->n_colliders < 0 || d->n_colliders > RVH_MAX_COLLIDERS || (d->n_colliders > 0 && !d->colliders))
        return fail(RVH_ERR_INVALID_ARG, "step_noalloc: at most 8 colliders");
    if (d->math != RVH_MATH_FAST && d->math != RVH_MATH_EXACT)
        return fail(RVH_ERR_INVALID_ARG, "step_noalloc: unknown math mode");
    rvh_status st = validate_params(*d->params);
    if (st != RVH_OK) return st;
    if ((st = validate_frame(*frame)) != RVH_OK) return st;
    const rvh_sim_params& P = *d->params;
    size_t cells = 0;
    if (P.grid_enabled) {
        cells = size_t(P.grid_dims[0]) * P.grid_dims[1] * P.grid_dims[2];
        if (cells > size_t(RVH_NOALLOC_MAX_GRID_CELLS))
            return fail(RVH_ERR_INVALID_ARG, "step_noalloc: the grid has more than RVH_NOALLOC_MAX_GRID_CELLS "
                                             "(64^3) cells; use rvh_step with an asset instead");
    }
    for (int j = 0; j < d->n_colliders; ++j)
        if (d->colliders[j].kind != RVH_COLLIDER_SPHERE && d->colliders[j].kind != RVH_COLLIDER_ELLIPSOID)
            return fail(RVH_ERR_INVALID_ARG, "step_noalloc: unknown collider kind");
    const int lanes = d->lanes_per_strand ? d->lanes_per_strand : default_lanes(d->n_points);
    const bool exact = d->math == RVH_MATH_EXACT;
    const void* ka = plain_a_kernel(d->n_points, lanes, exact);
    const void* kb = plain_b_kernel(exact);
    if (!ka) return fail(RVH_ERR_UNSUPPORTED, "step_noalloc: no phase-A kernel for this (n_points, lanes_per_strand)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (d->n_strands == 0) {   // nothing to step; the draw record still reports zero strands
        if (d->draw_indirect) {
            k_noalloc_empty_draw<<<1, 1, 0, s>>>(static_cast<rvh_draw_indirect*>(d->draw_indirect));
            RVH_CUDA(cudaGetLastError());
        }
        return RVH_OK;
    }
    int dev = 0;
    RVH_CUDA(cudaGetDevice(&dev));
    void* grid = nullptr;
    if ((st = scratch_address(dev, &grid)) != RVH_OK) return st;
    if (!prepare_kernel(ka) || !prepare_kernel(kb))
        return fail(RVH_ERR_CUDA, "step_noalloc: cannot opt the step kernels into shared memory");

    DevAsset A{};
    A.strands = static_cast<float4*>(d->strands);
    A.rest = d->rest_lengths;
    A.strand_wind = reinterpret_cast<const float4*>(d->strand_wind);
    A.grid = P.grid_enabled ? static_cast<unsigned long long*>(grid) : nullptr;
    A.draw = static_cast<rvh_draw_indirect*>(d->draw_indirect);
    A.n_strands = d->n_strands;
    A.n_points = d->n_points;
    for (int i = 0; i < 3; ++i) A.gravity[i] = P.gravity[i];
    A.damping = P.damping;
    A.dftl = P.dftl_damping;
    A.vmax = P.vmax;
    A.k_penalty = P.k_penalty;
    A.friction = P.friction;
    A.repulsion = P.repulsion;
    A.scale = P.grid_scale;
    A.grid_enabled = P.grid_enabled ? 1 : 0;
    A.wrap32 = P.grid_wrap32 ? 1 : 0;
    for (int i = 0; i < 3; ++i) A.origin[i] = P.grid_origin[i];
    A.h = P.grid_h;
    A.inv_h = 1.0f / P.grid_h;
    A.nx = P.grid_dims[0];
    A.ny = P.grid_dims[1];
    A.nz = P.grid_dims[2];
    A.dt = frame->dt;
    A.t = frame->t;
    for (int i = 0; i < 3; ++i) A.wind[i] = frame->wind[i];
    A.n_colliders = d->n_colliders;
    for (int j = 0; j < d->n_colliders; ++j) A.col[j] = pack_collider(d->colliders[j]);

    // the shared scratch keeps the previous call's sums: clear the cells this call uses
    if (P.grid_enabled) RVH_CUDA(cudaMemsetAsync(grid, 0, cells * 32u, s));
    void* args[] = {&A};
    const int per_cta = kWarps * (32 / lanes);
    const unsigned blocks_a = unsigned((d->n_strands + per_cta - 1) / per_cta);
    RVH_CUDA(cudaLaunchKernel(ka, dim3(blocks_a), dim3(kThreads), args, kSmemBytes, s));
    if (P.grid_enabled) {
        int sms = 0;
        RVH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const long long pts = (long long)d->n_strands * d->n_points;
        long long blocks = (pts + kTileB - 1) / kTileB;
        blocks = std::max(1LL, std::min(blocks, (long long)sms * 16));
        RVH_CUDA(cudaLaunchKernel(kb, dim3(unsigned(blocks)), dim3(kThreads), args, kSmemBytes, s));
    }
    return RVH_OK;
}

}  // extern "C"
