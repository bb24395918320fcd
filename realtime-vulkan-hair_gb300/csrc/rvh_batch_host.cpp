// rvh_batch_host.cpp — batched stepping: many assets advance in ONE persistent
// kernel launch, captured once in a CUDA graph and replayed every step.
//
// The plan is a queue of work items in dependency order.  For each asset
// (largest first): its phase-A strand tiles, then the clear of its other grid
// buffer (for the next step); its phase-B tiles are queued only after `lag`
// more items, so by the time a CTA pulls one the asset's phase A has almost
// always finished and the bounded wait in the kernel returns at once.
#include <algorithm>
#include <cstring>
#include <deque>
#include <new>

#include "rvh_internal.hpp"
#include "rvh_registry.h"

namespace rvh {

struct Batch {
    Context* ctx = nullptr;
    std::vector<Asset*> assets;
    int lanes = 4;
    bool exact = false;
    bool use_graph = true;
    int n_ctas = 0;
    int64_t n_points = 0;
    std::vector<WorkItem> items;
    std::vector<unsigned> need_a;
    DevBuf d_assets, d_items, d_need, d_done, d_head, d_error, d_stats;
    DevAsset* h_stage[2] = {nullptr, nullptr};
    cudaEvent_t staged[2] = {nullptr, nullptr};
    int slot = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BatchDev dev{};
    const void* kernel = nullptr;
    bool timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pairs;   // recorded, not yet read
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_free;
};

namespace {

constexpr int kTargetPointsA = 4096;   // points per phase-A item
constexpr int kTargetPointsB = kTileB;  // points per phase-B item (one shared-memory box)
constexpr int kClearChunk = 1 << 16;   // 16-B units per clear item (1 MiB)
constexpr uint32_t kSpinLimit = 1u << 22;  // ~1 s of 256-ns sleeps before a wait gives up

void plan(Batch& b, int strands_per_tile) {
    const int S = 32 / b.lanes;
    const int quantum = kWarps * S;
    std::vector<int> order(b.assets.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = int(i);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return int64_t(b.assets[x]->n_strands) * b.assets[x]->n_points >
               int64_t(b.assets[y]->n_strands) * b.assets[y]->n_points;
    });
    b.items.clear();
    b.need_a.assign(b.assets.size(), 0u);
    const size_t lag = size_t(2) * size_t(std::max(1, b.n_ctas));
    struct Pending {
        int asset;
        size_t last;
    };
    std::deque<Pending> pending;
    auto emit_b = [&](int ai) {
        const Asset* a = b.assets[ai];
        if (!a->params.grid_enabled) return;
        const int tb = std::max(1, kTargetPointsB / a->n_points);
        for (int s = 0; s < a->n_strands; s += tb) b.items.push_back({ITEM_B, ai, s, std::min(a->n_strands, s + tb)});
    };
    auto flush = [&](bool all) {
        while (!pending.empty() && (all || b.items.size() - pending.front().last >= lag)) {
            emit_b(pending.front().asset);
            pending.pop_front();
        }
    };
    for (int ai : order) {
        const Asset* a = b.assets[ai];
        if (a->n_strands == 0) continue;
        int ta = strands_per_tile > 0 ? strands_per_tile : kTargetPointsA / a->n_points;
        ta = std::max(quantum, (ta + quantum - 1) / quantum * quantum);
        for (int s = 0; s < a->n_strands; s += ta) {
            b.items.push_back({ITEM_A, ai, s, std::min(a->n_strands, s + ta)});
            b.need_a[ai]++;
            flush(false);
        }
        const size_t last = b.items.size();
        if (a->params.grid_enabled) {
            const int chunks = int(a->grid_bytes() / 16);
            for (int c = 0; c < chunks; c += kClearChunk)
                b.items.push_back({ITEM_CLEAR, ai, c, std::min(chunks, c + kClearChunk)});
        }
        pending.push_back({ai, last});
    }
    flush(true);
}

void destroy(Batch* b) {
    if (!b) return;
    if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
    for (auto& e : b->ev_pairs) cudaEventDestroy(e.first), cudaEventDestroy(e.second);
    for (auto& e : b->ev_free) cudaEventDestroy(e.first), cudaEventDestroy(e.second);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (int i = 0; i < 2; ++i) {
        if (b->staged[i]) cudaEventSynchronize(b->staged[i]), cudaEventDestroy(b->staged[i]);
        if (b->h_stage[i]) cudaFreeHost(b->h_stage[i]);
    }
    if (b->ctx) {
        b->ctx->free(b->d_assets);
        b->ctx->free(b->d_items);
        b->ctx->free(b->d_need);
        b->ctx->free(b->d_done);
        b->ctx->free(b->d_head);
        b->ctx->free(b->d_error);
        b->ctx->free(b->d_stats);
    }
    delete b;
}

rvh_status enqueue_launch(Batch* b, cudaStream_t s) {
    RVH_CUDA(cudaMemsetAsync(b->d_head.ptr, 0, sizeof(unsigned), s));
    RVH_CUDA(cudaMemsetAsync(b->d_done.ptr, 0, sizeof(unsigned) * b->assets.size(), s));
    void* args[] = {&b->dev};
    RVH_CUDA(cudaLaunchKernel(b->kernel, dim3(unsigned(b->n_ctas)), dim3(kThreads), args, kSmemBytes, s));
    return RVH_OK;
}

}  // namespace

// ---- dynamic batches (used by the request server) ---------------------------------
// The asset set changes from launch to launch: the plan and the per-asset
// tables are rebuilt and uploaded before each launch (no graph).
struct DynBatch {
    Batch b;
    size_t cap_assets = 0, cap_items = 0;
    WorkItem* h_items[2] = {nullptr, nullptr};
    unsigned* h_need[2] = {nullptr, nullptr};
};

static rvh_status dyn_reserve(DynBatch* d, size_t na, size_t ni) {
    Batch& b = d->b;
    if (na <= d->cap_assets && ni <= d->cap_items) return RVH_OK;
    RVH_CUDA(cudaStreamSynchronize(b.ctx->stream));
    for (int i = 0; i < 2; ++i) {
        if (b.staged[i]) RVH_CUDA(cudaEventSynchronize(b.staged[i]));
    }
    const size_t ca = std::max(na, d->cap_assets * 2 + 1), ci = std::max(ni, d->cap_items * 2 + 1);
    b.ctx->free(b.d_assets);
    b.ctx->free(b.d_items);
    b.ctx->free(b.d_need);
    b.ctx->free(b.d_done);
    rvh_status s;
    if ((s = b.ctx->alloc(b.d_assets, sizeof(DevAsset) * ca)) != RVH_OK) return s;
    if ((s = b.ctx->alloc(b.d_items, sizeof(WorkItem) * ci)) != RVH_OK) return s;
    if ((s = b.ctx->alloc(b.d_need, sizeof(unsigned) * ca)) != RVH_OK) return s;
    if ((s = b.ctx->alloc(b.d_done, sizeof(unsigned) * ca)) != RVH_OK) return s;
    for (int i = 0; i < 2; ++i) {
        if (b.h_stage[i]) cudaFreeHost(b.h_stage[i]);
        if (d->h_items[i]) cudaFreeHost(d->h_items[i]);
        if (d->h_need[i]) cudaFreeHost(d->h_need[i]);
        b.h_stage[i] = nullptr;
        d->h_items[i] = nullptr;
        d->h_need[i] = nullptr;
        RVH_CUDA(cudaMallocHost(&b.h_stage[i], sizeof(DevAsset) * ca));
        RVH_CUDA(cudaMallocHost(&d->h_items[i], sizeof(WorkItem) * ci));
        RVH_CUDA(cudaMallocHost(&d->h_need[i], sizeof(unsigned) * ca));
    }
    d->cap_assets = ca;
    d->cap_items = ci;
    b.dev.assets = static_cast<const DevAsset*>(b.d_assets.ptr);
    b.dev.items = static_cast<const WorkItem*>(b.d_items.ptr);
    b.dev.done_a = static_cast<unsigned*>(b.d_done.ptr);
    b.dev.need_a = static_cast<const unsigned*>(b.d_need.ptr);
    return RVH_OK;
}

DynBatch* dyn_batch_new(Context* ctx, int lanes, rvh_status* st) {
    *st = RVH_OK;
    if (!batch_supported(lanes)) {
        *st = fail(RVH_ERR_UNSUPPORTED, "lanes_per_strand must be 4, 8, 16 or 32");
        return nullptr;
    }
    DynBatch* d = new (std::nothrow) DynBatch();
    if (!d) {
        *st = fail(RVH_ERR_OUT_OF_MEMORY, "host allocation failed");
        return nullptr;
    }
    Batch& b = d->b;
    b.ctx = ctx;
    b.lanes = lanes;
    b.exact = ctx->math == RVH_MATH_EXACT;
    b.use_graph = false;
    b.kernel = batch_kernel(lanes, b.exact);
    int per_sm = 0;
    if (!prepare_kernel(b.kernel) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b.kernel, kThreads, kSmemBytes) != cudaSuccess) {
        *st = fail(RVH_ERR_CUDA, "cannot prepare the batch kernel");
        delete d;
        return nullptr;
    }
    b.n_ctas = std::max(1, per_sm) * ctx->sm_count;
    rvh_status s;
    if ((s = ctx->alloc(b.d_head, sizeof(unsigned))) != RVH_OK || (s = ctx->alloc(b.d_error, sizeof(int))) != RVH_OK ||
        (s = ctx->alloc(b.d_stats, 4 * sizeof(unsigned))) != RVH_OK) {
        *st = s;
        dyn_batch_free(d);
        return nullptr;
    }
    cudaMemset(b.d_error.ptr, 0, sizeof(int));
    cudaMemset(b.d_stats.ptr, 0, 4 * sizeof(unsigned));
    for (int i = 0; i < 2; ++i) cudaEventCreateWithFlags(&b.staged[i], cudaEventDisableTiming);
    b.dev.spin_limit = kSpinLimit;
    b.dev.head = static_cast<unsigned*>(b.d_head.ptr);
    b.dev.error = static_cast<int*>(b.d_error.ptr);
    b.dev.stats = static_cast<unsigned*>(b.d_stats.ptr);
    return d;
}

void dyn_batch_free(DynBatch* d) {
    if (!d) return;
    for (int i = 0; i < 2; ++i) {
        if (d->h_items[i]) cudaFreeHost(d->h_items[i]);
        if (d->h_need[i]) cudaFreeHost(d->h_need[i]);
        d->h_items[i] = nullptr;
        d->h_need[i] = nullptr;
    }
    Batch* b = new Batch();
    *b = d->b;      // hand the buffers to the common destructor
    d->b = Batch();
    destroy(b);
    delete d;
}

rvh_status dyn_batch_launch(DynBatch* d, const std::vector<Asset*>& assets, const std::vector<rvh_frame>& frames,
                            cudaStream_t s, cudaEvent_t ev_start, cudaEvent_t ev_stop, int64_t* points) {
    Batch& b = d->b;
    b.assets = assets;
    plan(b, 0);
    b.dev.n_items = int32_t(b.items.size());
    int64_t pts = 0;
    for (Asset* a : assets) pts += int64_t(a->n_strands) * a->n_points;
    if (points) *points = pts;
    if (b.items.empty()) return RVH_OK;
    rvh_status st = dyn_reserve(d, assets.size(), b.items.size());
    if (st != RVH_OK) return st;
    const int slot = b.slot;
    b.slot ^= 1;
    RVH_CUDA(cudaEventSynchronize(b.staged[slot]));
    for (size_t i = 0; i < assets.size(); ++i) {
        Asset* a = assets[i];
        if (a->params.grid_enabled && a->grid_dirty[a->parity])
            RVH_CUDA(cudaMemsetAsync(a->grid[a->parity].ptr, 0, a->grid_bytes(), s));
        b.h_stage[slot][i] = a->device_view(frames[i], a->parity);
        d->h_need[slot][i] = b.need_a[i];
    }
    std::memcpy(d->h_items[slot], b.items.data(), sizeof(WorkItem) * b.items.size());
    RVH_CUDA(cudaMemcpyAsync(b.d_assets.ptr, b.h_stage[slot], sizeof(DevAsset) * assets.size(), cudaMemcpyHostToDevice, s));
    RVH_CUDA(cudaMemcpyAsync(b.d_items.ptr, d->h_items[slot], sizeof(WorkItem) * b.items.size(), cudaMemcpyHostToDevice, s));
    RVH_CUDA(cudaMemcpyAsync(b.d_need.ptr, d->h_need[slot], sizeof(unsigned) * assets.size(), cudaMemcpyHostToDevice, s));
    RVH_CUDA(cudaEventRecord(b.staged[slot], s));
    if (ev_start) RVH_CUDA(cudaEventRecord(ev_start, s));
    rvh_status ls = enqueue_launch(&b, s);
    if (ls != RVH_OK) return ls;
    if (ev_stop) RVH_CUDA(cudaEventRecord(ev_stop, s));
    for (Asset* a : assets) {
        if (!a->params.grid_enabled) continue;
        a->grid_dirty[a->parity] = true;
        a->grid_dirty[a->parity ^ 1] = false;
        a->parity ^= 1;
    }
    return RVH_OK;
}

rvh_status dyn_batch_check(DynBatch* d) {
    int err = 0;
    RVH_CUDA(cudaMemcpy(&err, d->b.d_error.ptr, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        cudaMemset(d->b.d_error.ptr, 0, sizeof(int));
        return fail(err, "server batch: a phase-B tile gave up waiting for its asset's phase A");
    }
    return RVH_OK;
}

int dyn_batch_ctas(const DynBatch* d) { return d->b.n_ctas; }

}  // namespace rvh

struct rvh_batch : rvh::Batch {};

using namespace rvh;

extern "C" {

rvh_status rvh_batch_create(rvh_context* ctx, rvh_asset* const* assets, int32_t n, const rvh_batch_desc* desc,
                            rvh_batch** out) {
    if (!ctx || !out || (n > 0 && !assets) || n < 0) return fail(RVH_ERR_INVALID_ARG, "batch_create: bad argument");
    *out = nullptr;
    rvh_batch_desc d{};
    d.use_graph = 1;
    if (desc) d = *desc;
    int lanes = d.lanes_per_strand;
    if (lanes == 0) {  // the tuner's choice for this workload, if it has one
        rvh_tune_result tr{};
        const std::string keep = last_error_cstr();
        if (n > 0 && rvh_tune_lookup(assets, n, 0, &tr) == RVH_OK) {
            lanes = tr.lanes_per_strand;
            if (d.strands_per_tile == 0) d.strands_per_tile = tr.strands_per_tile;
        } else {
            lanes = 4;
        }
        set_error(keep);
    }
    if (!batch_supported(lanes)) return fail(RVH_ERR_UNSUPPORTED, "batch: lanes_per_strand must be 4, 8, 16 or 32");
    cudaSetDevice(ctx->device);
    rvh_batch* b = new (std::nothrow) rvh_batch();
    if (!b) return fail(RVH_ERR_OUT_OF_MEMORY, "host allocation failed");
    b->ctx = ctx;
    b->lanes = lanes;
    b->exact = ctx->math == RVH_MATH_EXACT;
    b->use_graph = d.use_graph != 0;
    for (int i = 0; i < n; ++i) {
        if (!assets[i] || assets[i]->ctx != ctx) {
            destroy(b);
            return fail(RVH_ERR_INVALID_ARG, "batch_create: every asset must belong to this context");
        }
        for (int j = 0; j < i; ++j)
            if (assets[j] == assets[i]) {
                destroy(b);
                return fail(RVH_ERR_INVALID_ARG, "batch_create: an asset appears twice");
            }
        b->assets.push_back(assets[i]);
        b->n_points += int64_t(assets[i]->n_strands) * assets[i]->n_points;
    }
    b->kernel = batch_kernel(lanes, b->exact);
    if (!prepare_kernel(b->kernel)) {
        destroy(b);
        return fail(RVH_ERR_CUDA, "cannot opt the batch kernel into shared memory");
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->kernel, kThreads, kSmemBytes);
    if (e != cudaSuccess) {
        destroy(b);
        return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    }
    if (d.ctas_per_sm > 0) per_sm = std::min(per_sm, int(d.ctas_per_sm));
    b->n_ctas = std::max(1, per_sm) * ctx->sm_count;
    plan(*b, d.strands_per_tile);
    rvh_status s;
    auto bail = [&](rvh_status st) {
        destroy(b);
        return st;
    };
    const size_t na = std::max<size_t>(1, b->assets.size());
    if ((s = ctx->alloc(b->d_assets, sizeof(DevAsset) * na)) != RVH_OK) return bail(s);
    if ((s = ctx->alloc(b->d_items, sizeof(WorkItem) * std::max<size_t>(1, b->items.size()))) != RVH_OK) return bail(s);
    if ((s = ctx->alloc(b->d_need, sizeof(unsigned) * na)) != RVH_OK) return bail(s);
    if ((s = ctx->alloc(b->d_done, sizeof(unsigned) * na)) != RVH_OK) return bail(s);
    if ((s = ctx->alloc(b->d_head, sizeof(unsigned))) != RVH_OK) return bail(s);
    if ((s = ctx->alloc(b->d_error, sizeof(int))) != RVH_OK) return bail(s);
    if ((s = ctx->alloc(b->d_stats, 4 * sizeof(unsigned))) != RVH_OK) return bail(s);
    e = cudaMemset(b->d_stats.ptr, 0, 4 * sizeof(unsigned));
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemset stats"));
    if (!b->items.empty()) {
        e = cudaMemcpy(b->d_items.ptr, b->items.data(), sizeof(WorkItem) * b->items.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy items"));
    }
    if (!b->need_a.empty()) {
        e = cudaMemcpy(b->d_need.ptr, b->need_a.data(), sizeof(unsigned) * b->need_a.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy need"));
    }
    e = cudaMemset(b->d_error.ptr, 0, sizeof(int));
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemset error"));
    for (int i = 0; i < 2; ++i) {
        e = cudaMallocHost(&b->h_stage[i], sizeof(DevAsset) * na);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMallocHost"));
        e = cudaEventCreateWithFlags(&b->staged[i], cudaEventDisableTiming);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaEventCreate"));
    }
    b->dev.assets = static_cast<const DevAsset*>(b->d_assets.ptr);
    b->dev.items = static_cast<const WorkItem*>(b->d_items.ptr);
    b->dev.n_items = int32_t(b->items.size());
    b->dev.spin_limit = kSpinLimit;
    b->dev.head = static_cast<unsigned*>(b->d_head.ptr);
    b->dev.done_a = static_cast<unsigned*>(b->d_done.ptr);
    b->dev.need_a = static_cast<const unsigned*>(b->d_need.ptr);
    b->dev.error = static_cast<int*>(b->d_error.ptr);
    b->dev.stats = static_cast<unsigned*>(b->d_stats.ptr);
    if (b->use_graph && !b->items.empty()) {
        cudaStream_t cs = ctx->stream;
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamBeginCapture"));
        rvh_status ls = enqueue_launch(b, cs);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(cs, &g);
        if (ls != RVH_OK) {
            if (g) cudaGraphDestroy(g);
            return bail(ls);
        }
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamEndCapture"));
        b->graph = g;
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaGraphInstantiate"));
    }
    *out = b;
    return RVH_OK;
}

rvh_status rvh_batch_destroy(rvh_batch* b) {
    destroy(b);
    return RVH_OK;
}

rvh_status rvh_batch_step(rvh_batch* b, const rvh_frame* frames, void* stream) {
    if (!b || (!frames && !b->assets.empty())) return fail(RVH_ERR_INVALID_ARG, "batch_step: NULL argument");
    for (size_t i = 0; i < b->assets.size(); ++i) {
        rvh_status s = validate_frame(frames[i]);
        if (s != RVH_OK) return s;
    }
    if (b->items.empty()) return RVH_OK;
    cudaSetDevice(b->ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->ctx->stream;
    const int slot = b->slot;
    b->slot ^= 1;
    RVH_CUDA(cudaEventSynchronize(b->staged[slot]));  // the copy that last read this staging buffer is done
    DevAsset* st = b->h_stage[slot];
    for (size_t i = 0; i < b->assets.size(); ++i) {
        Asset* a = b->assets[i];
        if (a->params.grid_enabled && a->grid_dirty[a->parity])  // left dirty by a plain step
            RVH_CUDA(cudaMemsetAsync(a->grid[a->parity].ptr, 0, a->grid_bytes(), s));
        st[i] = a->device_view(frames[i], a->parity);
    }
    RVH_CUDA(cudaMemcpyAsync(b->d_assets.ptr, st, sizeof(DevAsset) * b->assets.size(), cudaMemcpyHostToDevice, s));
    RVH_CUDA(cudaEventRecord(b->staged[slot], s));
    std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
    if (b->timing) {
        if (!b->ev_free.empty()) {
            ev = b->ev_free.back();
            b->ev_free.pop_back();
        } else {
            RVH_CUDA(cudaEventCreate(&ev.first));
            RVH_CUDA(cudaEventCreate(&ev.second));
        }
        RVH_CUDA(cudaEventRecord(ev.first, s));
    }
    if (b->exec) {
        RVH_CUDA(cudaGraphLaunch(b->exec, s));
    } else {
        rvh_status ls = enqueue_launch(b, s);
        if (ls != RVH_OK) return ls;
    }
    if (b->timing) {
        RVH_CUDA(cudaEventRecord(ev.second, s));
        b->ev_pairs.push_back(ev);
    }
    for (Asset* a : b->assets) {
        if (!a->params.grid_enabled) continue;
        a->grid_dirty[a->parity] = true;       // used by this step (read back by rvh_asset_read_grid)
        a->grid_dirty[a->parity ^ 1] = false;  // cleared by this step
        a->parity ^= 1;
    }
    return RVH_OK;
}

rvh_status rvh_batch_check(rvh_batch* b) {
    if (!b) return fail(RVH_ERR_INVALID_ARG, "batch_check: NULL");
    cudaSetDevice(b->ctx->device);
    RVH_CUDA(cudaStreamSynchronize(b->ctx->stream));
    RVH_CUDA(cudaDeviceSynchronize());
    int err = 0;
    RVH_CUDA(cudaMemcpy(&err, b->d_error.ptr, sizeof(int), cudaMemcpyDeviceToHost));
    if (err != 0) {
        RVH_CUDA(cudaMemset(b->d_error.ptr, 0, sizeof(int)));
        return fail(err, "batch: a phase-B tile gave up waiting for its asset's phase A");
    }
    return RVH_OK;
}

rvh_status rvh_batch_h2d_bytes(rvh_batch* b, uint64_t* bytes) {
    if (!b || !bytes) return fail(RVH_ERR_INVALID_ARG, "batch_h2d_bytes: NULL");
    *bytes = uint64_t(sizeof(DevAsset)) * b->assets.size();
    return RVH_OK;
}

rvh_status rvh_batch_timing_enable(rvh_batch* b, int32_t on) {
    if (!b) return fail(RVH_ERR_INVALID_ARG, "batch_timing_enable: NULL");
    b->timing = on != 0;
    return RVH_OK;
}

rvh_status rvh_batch_timing_read(rvh_batch* b, double* total_ms, int32_t* launches) {
    if (!b) return fail(RVH_ERR_INVALID_ARG, "batch_timing_read: NULL");
    double sum = 0.0;
    for (auto& e : b->ev_pairs) {
        RVH_CUDA(cudaEventSynchronize(e.second));
        float ms = 0.f;
        RVH_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
        sum += ms;
        b->ev_free.push_back(e);
    }
    if (launches) *launches = int32_t(b->ev_pairs.size());
    if (total_ms) *total_ms = sum;
    b->ev_pairs.clear();
    return RVH_OK;
}

rvh_status rvh_batch_box_stats(rvh_batch* b, uint32_t out[4]) {
    if (!b || !out) return fail(RVH_ERR_INVALID_ARG, "batch_box_stats: NULL");
    cudaSetDevice(b->ctx->device);
    RVH_CUDA(cudaStreamSynchronize(b->ctx->stream));
    RVH_CUDA(cudaMemcpy(out, b->d_stats.ptr, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost));
    RVH_CUDA(cudaMemset(b->d_stats.ptr, 0, 4 * sizeof(unsigned)));
    return RVH_OK;
}

rvh_status rvh_batch_info(rvh_batch* b, int32_t* lanes, int32_t* n_items, int32_t* n_ctas, int64_t* n_points) {
    if (!b) return fail(RVH_ERR_INVALID_ARG, "batch_info: NULL");
    if (lanes) *lanes = b->lanes;
    if (n_items) *n_items = int32_t(b->items.size());
    if (n_ctas) *n_ctas = b->n_ctas;
    if (n_points) *n_points = b->n_points;
    return RVH_OK;
}

}  // extern "C"
