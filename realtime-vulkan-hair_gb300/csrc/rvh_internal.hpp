// rvh_internal.hpp — host-side objects behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rvh.h"
#include "rvh_kernels.cuh"

#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>   // header-only NVTX v3: a no-op unless a profiler is attached
#define RVH_HAVE_NVTX 1
#else
#define RVH_HAVE_NVTX 0
#endif

namespace rvh {

// ---- errors -------------------------------------------------------------------
void set_error(const std::string& msg);
const char* last_error_cstr();
rvh_status fail(rvh_status s, const std::string& msg);
rvh_status cuda_fail(cudaError_t e, const char* what);
#define RVH_CUDA(call)                                              \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return ::rvh::cuda_fail(e_, #call);  \
    } while (0)

// Makes `dev` current for the guard's lifetime and puts the caller's device
// back afterwards, so no entry point leaks a device switch into host code
// that drives several GPUs.  RVH_DEVICE(dev) declares one and returns the
// CUDA error when the switch fails.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};
#define RVH_DEVICE(dev)                                                                         \
    ::rvh::DeviceGuard rvh_device_guard_(dev);                                                  \
    if (rvh_device_guard_.err != cudaSuccess) return ::rvh::cuda_fail(rvh_device_guard_.err, "cudaSetDevice")

// ---- HBM admission accounting --------------------------------------------------
// Every device allocation a context makes is admitted against its budget
// first; a request that would exceed it fails with RVH_ERR_BUDGET and
// allocates nothing.
class Budget {
public:
    void init(uint64_t budget) { budget_ = budget; }
    bool reserve(uint64_t bytes) {
        uint64_t cur = used_.load();
        do {
            if (cur + bytes > budget_) return false;
        } while (!used_.compare_exchange_weak(cur, cur + bytes));
        return true;
    }
    void release(uint64_t bytes) { used_.fetch_sub(bytes); }
    uint64_t used() const { return used_.load(); }
    uint64_t budget() const { return budget_; }

private:
    uint64_t budget_ = 0;
    std::atomic<uint64_t> used_{0};
};

struct Context;

// An NVTX range around a public entry point, for timeline tools (nsys, ncu --nvtx).
struct TraceRange {
    explicit TraceRange(const char* name) {
#if RVH_HAVE_NVTX
        nvtxRangePushA(name);
#else
        (void)name;
#endif
    }
    ~TraceRange() {
#if RVH_HAVE_NVTX
        nvtxRangePop();
#endif
    }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// A device allocation charged to a context's budget.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    Context* owner = nullptr;
    bool owned = true;
};

struct Context {
    int device = 0;
    int math = RVH_MATH_FAST;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    Budget budget;
    std::mutex mu;

    rvh_status alloc(DevBuf& b, size_t bytes);
    void free(DevBuf& b);
};

struct Asset {
    Context* ctx = nullptr;
    int n_strands = 0;
    int n_points = 0;
    int lanes = 0;
    DevBuf strands;   // borrowed when created with RVH_MEM_DEVICE_BORROWED
    DevBuf rest;
    DevBuf wind;      // float4 per strand, or empty
    DevBuf grid[3];   // 4 x int64 per cell; a fused batched step gathers from one, splats into
                      // another and clears the third
    DevBuf draw;
    bool grid_dirty[3] = {false, false, false};
    // Fused batched steps leave the last step's gather + friction (loop 3) pending: positions
    // are final, velocities still lack the friction blend, which the next fused step (or a
    // finish) applies from grid[pend] with dt_prev.
    bool pending = false;
    int pend = 0;
    float dt_prev = 0.f;
    int last_grid = -1;         // grid of the most recent splat (rvh_asset_read_grid)
    size_t grid_cells = 0;
    rvh_sim_params params{};
    std::vector<rvh_collider> colliders;
    bool has_wind = false;
    bool server_managed = false;  // grids are lent by a request server while a request is active
    // grid group (rvh_asset_share_grid): a member's grid[] alias its owner's buffers (not owned);
    // the owner keeps the group's grid state (which buffer is pending, dirty) and its members
    Asset* grid_owner = nullptr;
    std::vector<Asset*> grid_members;
    bool grid_grouped() const { return grid_owner != nullptr || !grid_members.empty(); }
    // kinematic head (rvh_asset_set_head_transform): roots = head * root_rest each step
    bool head_active = false;
    float head[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};   // column-major
    DevBuf root_rest;   // float4 per strand, captured at the first head transform
    // phase-A group boxes a fused batched step leaves for the next one (DevAsset::group_box):
    // the tag of the last write and the grouping (lanes, strands per tile) it was written with
    DevBuf group_boxes;
    uint32_t box_tag = 0;
    uint32_t box_layout = 0;
    // tessellation tables of the last descriptor (rvh_asset_tessellate)
    DevBuf tess_tables;
    DevBuf tess_cache;   // per strand: root bits and the sd profiles computed from them
    // rvh_asset_render_hair's blending scratch: per-pixel counts, offsets, cursors and tile sums;
    // the per-pixel fragment lists; the rasterising passes' list of near-clipped quads
    DevBuf raster_px, raster_frags, raster_clip;
    rvh_tess_desc tess_desc{};
    size_t tess_off[6] = {0, 0, 0, 0, 0, 0};

    size_t record_bytes() const { return size_t(n_strands) * 48u * size_t(n_points); }
    size_t grid_bytes() const { return grid_cells * 32u; }
    // DevAsset for one step with frame f: splat into / gather from grid[g], gather the pending
    // friction from grid[prev] (or none: -1), clear grid[next] (or none: -1).
    DevAsset device_view(const rvh_frame& f, int g, int prev = -1, int next = -1) const;
    // A clean grid index other than the two given (-1 = none); dirty ones only if no clean one.
    int pick_grid(int avoid1, int avoid2) const;
};

rvh_status validate_params(const rvh_sim_params& p);
rvh_status validate_frame(const rvh_frame& f);
DevCollider pack_collider(const rvh_collider& c);
// rest carried by the head motion m (column-major affine): transform = m * rest.transform
bool follow_collider(const rvh_collider& rest, const float* m, rvh_collider* out);
int default_lanes(int n_points);
rvh_status ensure_grid(Asset* a);
rvh_status launch_plain(Asset* a, const rvh_frame& f, cudaStream_t s);
// Applies a pending friction (gather-only pass on grid[pend]); no-op when none is pending.
rvh_status finish_pending(Asset* a, cudaStream_t s);

// Batches whose asset set changes per launch (rvh_batch_host.cpp).
struct DynBatch;
DynBatch* dyn_batch_new(Context* ctx, int lanes, rvh_status* st);
void dyn_batch_free(DynBatch* d);
// modes: 0 = fused (the step's loop 3 stays pending), 1 = full step (loop 3 in the same launch)
rvh_status dyn_batch_launch(DynBatch* d, const std::vector<Asset*>& assets, const std::vector<rvh_frame>& frames,
                            const std::vector<int>& modes, cudaStream_t s, cudaEvent_t ev_start, cudaEvent_t ev_stop,
                            int64_t* points);
// Several fused steps per asset in one launch (steps[i]; frames: per asset its steps' frames);
// mode 2 (finish) entries take one step.
rvh_status dyn_batch_launch_steps(DynBatch* d, const std::vector<Asset*>& assets, const std::vector<int>& steps,
                                  const std::vector<int>& modes, const std::vector<rvh_frame>& frames, cudaStream_t s,
                                  cudaEvent_t ev_start, cudaEvent_t ev_stop);
rvh_status dyn_batch_check(DynBatch* d);
int dyn_batch_ctas(const DynBatch* d);

}  // namespace rvh

struct rvh_context : rvh::Context {};
struct rvh_asset : rvh::Asset {};
