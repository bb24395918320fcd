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

enum { MODE_FUSED = 0, MODE_FULL = 1, MODE_FINISH = 2 };

struct Batch {
    Context* ctx = nullptr;
    std::vector<Asset*> assets;
    std::vector<int> modes;   // per asset: MODE_FUSED (loop 3 left pending), MODE_FULL, MODE_FINISH
    std::vector<int> tile_strands;   // per asset: strands per phase-A item of the current plan
    std::vector<int> group_rounds;   // per asset: rounds per phase-A group of the current plan
    int min_tile_points = 0;         // > 0: groups no larger than this (a request server's small launches)
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
    // positions read-back: packed device staging (two slots) and a copy stream
    DevBuf pos_stage[2], d_first;   // staging slots; d_first: the pack kernel's chunk table
    int n_pack_chunks = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t packed[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    int pos_slot = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pairs;   // recorded, not yet read
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_free;
    DynBatch* finisher = nullptr;   // one launch of gather-only items for rvh_batch_finish
    std::vector<int64_t> first_point;   // per asset: its first point in the batch's position order
    // grid groups: per asset the batch index of its grid owner (itself for an owner with
    // members, -1 for an asset with a grid of its own)
    std::vector<int> grid_root;
    // several steps per launch (a request server's launches): per entry of `assets` the step
    // it is of its asset (empty: one step each); a step's entries form one segment of the queue
    std::vector<int> entry_step;
};

// Packs the curvePoints of every asset of a batch into one contiguous float4
// array (asset after asset): out[first[a] + s*n + i] = strands[s*3n + i].
// Packs curvePoints of whole strands into a contiguous staging buffer.
// Chunk c covers strands [strand0, strand0 + count) of asset `asset`, whose
// points start at `out0` in the output; one CTA per chunk (grid-stride),
// consecutive threads copy consecutive points (coalesced on both sides).
struct PackChunk {
    int asset, strand0, count, n;
    long long out0;
};

template <bool kXyz>
__global__ void __launch_bounds__(kThreads) k_pack_positions(const DevAsset* __restrict__ assets,
                                                             const PackChunk* __restrict__ chunks, int n_chunks,
                                                             void* __restrict__ out) {
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        const PackChunk ch = chunks[c];
        const float4* src = assets[ch.asset].strands + (size_t)ch.strand0 * (3 * ch.n);
        const int pts = ch.count * ch.n;
        const FastDiv dn((unsigned)ch.n);
        for (int q = threadIdx.x; q < pts; q += kThreads) {
            const int s = (int)dn.div((unsigned)q), i = q - s * ch.n;
            const float4 v = __ldcs(src + (size_t)s * (3 * ch.n) + i);
            if (kXyz) {
                float* o = static_cast<float*>(out) + 3 * (ch.out0 + q);
                o[0] = v.x;
                o[1] = v.y;
                o[2] = v.z;
            } else {
                static_cast<float4*>(out)[ch.out0 + q] = v;
            }
        }
    }
}

namespace {

constexpr int kTargetPointsA = 4096;   // points per phase-A item
constexpr int kMinTilePoints = 512;   // smallest phase-A item of a request-server launch
constexpr int kTargetPointsB = kTileB;  // points per phase-B item (one shared-memory box)
constexpr int kClearChunk = 1 << 16;   // 16-B units per clear item (1 MiB)
constexpr int kSparseCellsPerStrand = 50;   // grid cells per strand from which an asset's items go first
constexpr uint32_t kSpinLimit = 1u << 22;  // ~1 s of 256-ns sleeps before a wait gives up

// strands_per_tile > 0 fixes the phase-A tile; else a tile holds about
// target_points points (rounded to whole CTA rounds).
void plan(Batch& b, int strands_per_tile, int target_points = kTargetPointsA) {
    const int S = 32 / b.lanes;
    const int quantum = kWarps * S;
    std::vector<int> order(b.assets.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = int(i);
    // Sparse assets first: few strands over a large grid give every round a large, mostly
    // empty splat box (many shared-memory slabs), so their items take several times as long
    // per point (about 90 ns against 30 at 50+ cells per strand on the 256-head workload);
    // started last they were the launch's tail.  Then the rest grouped by points per strand
    // (CTAs then mostly run one unrolled code path at a time; mixing them cost 10 %), smallest
    // assets first inside a group, which leaves the short items of dense assets for the end.
    // (Several steps per launch: step by step, each step's entries in that order.)
    const bool multi = !b.entry_step.empty();
    auto step_of = [&](int i) { return multi ? b.entry_step[i] : 0; };
    auto sparse = [&](const Asset* a) {
        return a->params.grid_enabled && a->n_strands > 0 &&
               a->grid_cells >= size_t(kSparseCellsPerStrand) * size_t(a->n_strands);
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        if (step_of(x) != step_of(y)) return step_of(x) < step_of(y);
        const Asset* ax = b.assets[x];
        const Asset* ay = b.assets[y];
        const bool sx = sparse(ax), sy = sparse(ay);
        if (sx != sy) return sx;
        if (ax->n_points != ay->n_points) return ax->n_points > ay->n_points;
        return int64_t(ax->n_strands) * ax->n_points < int64_t(ay->n_strands) * ay->n_points;
    });
    b.items.clear();
    b.need_a.assign(b.assets.size(), 0u);
    b.tile_strands.assign(b.assets.size(), 0);
    b.group_rounds.assign(b.assets.size(), 0);
    const size_t lag = size_t(2) * size_t(std::max(1, b.n_ctas));
    struct Pending {
        int asset;
        size_t last;
    };
    std::deque<Pending> pending;
    std::vector<WorkItem> clears;
    std::vector<size_t> seg_items, seg_clears;   // per step: where its work items and clears start
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
    // The last two waves of phase-A work (about 2 x 1,024 points per CTA) go out in items of
    // one group: CTAs then finish within a short item of one another (with the launch's
    // own tiles of up to 4,096 points the 64-character launch's CTAs ended 200 us apart).
    int64_t a_left = 0;
    for (int ai : order) {
        const Asset* a = b.assets[ai];
        const int mode = b.modes.empty() ? MODE_FUSED : b.modes[ai];
        if (mode != MODE_FINISH) a_left += int64_t(a->n_strands) * a->n_points;
    }
    const int64_t taper = int64_t(2) * std::max(1, b.n_ctas) * (kTargetPointsA / 4);
    for (int ai : order) {
        const Asset* a = b.assets[ai];
        while (int(seg_items.size()) <= step_of(ai)) {
            seg_items.push_back(b.items.size());
            seg_clears.push_back(clears.size());
        }
        const bool owner = !b.grid_root.empty() && b.grid_root[ai] == ai;   // clears its group's grid
        if (a->n_strands == 0 && !owner) continue;
        const int mode = b.modes.empty() ? MODE_FUSED : b.modes[ai];
        if (mode == MODE_FINISH) {  // gather-only items of an earlier step: nothing to wait for
            emit_b(ai);
            continue;
        }
        // Rounds per group (the kernel's boxes span a group): at most kUnionRounds and fewer than
        // 4e9 / scale points, as the kernel computes it; a server keeps groups within its smallest
        // tile, so the grouping, and the boxes one step leaves the next, do not change from launch
        // to launch.  Tiles are whole groups, the nearest to target_points.
        const float cap = 4.0e9f / (a->params.grid_scale * float(quantum * a->n_points));
        int U = std::max(1, std::min(kUnionRounds, int(cap)));
        const int span = b.min_tile_points > 0 ? b.min_tile_points : target_points;   // groups fit a tile
        U = std::max(1, std::min(U, span / (quantum * a->n_points)));
        const int group = quantum * U;
        int ta;
        if (strands_per_tile > 0) {
            ta = std::max(quantum, (strands_per_tile + quantum - 1) / quantum * quantum);
        } else {
            const int want = std::max(1, target_points / a->n_points);
            ta = std::max(1, (want + group / 2) / group) * group;
        }
        b.tile_strands[ai] = ta;
        b.group_rounds[ai] = U;
        for (int s = 0; s < a->n_strands;) {
            const int e = std::min(a->n_strands, s + (a_left <= taper ? std::min(ta, group) : ta));
            b.items.push_back({ITEM_A, ai, s, e});
            b.need_a[ai]++;
            a_left -= int64_t(e - s) * a->n_points;
            s = e;
            flush(false);
        }
        const size_t last = b.items.size();
        const bool member = !b.grid_root.empty() && b.grid_root[ai] >= 0 && b.grid_root[ai] != ai;
        if (a->params.grid_enabled && !member) {   // a group's grid is cleared once, by its owner
            const int chunks = int(a->grid_bytes() / 16);
            for (int c = 0; c < chunks; c += kClearChunk) {
                clears.push_back({ITEM_CLEAR, ai, c, std::min(chunks, c + kClearChunk)});
                if (multi) b.need_a[ai]++;   // the asset's next step waits for its clears too
            }
        }
        if (mode == MODE_FULL) pending.push_back({ai, last});
    }
    flush(true);
    // The clears (of grids this launch does not read) spread evenly through the queue:
    // memory-bound work beside the compute, and none left for a tail at the end (one
    // large asset's clears after its last tile kept a few CTAs busy after the rest).
    // With several steps per launch each step's clears stay within its own segment, ahead
    // of every item of the next step (whose waits are then all on earlier items).
    if (!clears.empty()) {
        std::vector<WorkItem> merged;
        merged.reserve(b.items.size() + clears.size());
        seg_items.push_back(b.items.size());
        seg_clears.push_back(clears.size());
        for (size_t g = 0; g + 1 < seg_items.size(); ++g) {
            const size_t w0 = seg_items[g], nw = seg_items[g + 1] - w0;
            const size_t c0 = seg_clears[g], nc = seg_clears[g + 1] - c0;
            size_t wi = 0;
            for (size_t c = 0; c < nc; ++c) {
                const size_t upto = (c * nw) / nc;   // clear c goes before work item upto
                while (wi < upto) merged.push_back(b.items[w0 + wi++]);
                merged.push_back(clears[c0 + c]);
            }
            while (wi < nw) merged.push_back(b.items[w0 + wi++]);
        }
        b.items.swap(merged);
    }
    // the L2 prefetch of the next item pays for items of about 2,048 points and more
    int64_t a_items = 0, a_points = 0;
    for (const WorkItem& w : b.items)
        if (w.kind == ITEM_A) {
            ++a_items;
            a_points += int64_t(w.end - w.begin) * b.assets[w.asset]->n_points;
        }
    b.dev.prefetch = a_items > 0 && a_points >= 2048 * a_items ? 1 : 0;
    b.dev.count_clears = multi ? 1 : 0;
}

// Grid choice of one asset for one batched step: gather the pending friction from
// grid[prev], splat into grid[t] (cleared first if dirty), clear grid[u] in-kernel.
// box_tag: the group-box tag this launch writes (0: none).
struct GridUse {
    int prev = -1, t = -1, u = -1;
    uint32_t box_tag = 0;
};

// The grouping of an asset's phase-A rounds in a launch.  Groups are counted
// from each item's first round, so with items of whole groups they start at
// multiples of the group size whatever the tile: the grouping is (lanes per
// strand, rounds per group); otherwise it also depends on the tile.  One
// thread per strand (lanes 1) keeps no group boxes: 0.
uint32_t box_layout_of(const Batch& b, size_t i) {
    if (b.lanes <= 1) return 0u;
    const int quantum = kWarps * (32 / b.lanes), group = quantum * b.group_rounds[i];
    const uint32_t key = (uint32_t(b.lanes) << 24) | (uint32_t(b.group_rounds[i]) << 20);
    return b.tile_strands[i] % group == 0 ? key : key | (1u << 19) | uint32_t(b.tile_strands[i] & 0x7ffff);
}

// The asset's stored group boxes for this step's view (optional: without a record buffer every
// fused step recomputes its gather boxes).
void attach_group_boxes(Asset* a, DevAsset* view, GridUse* gu, uint32_t layout) {
    // one record pair per round of 8 strands at most (32 lanes per strand)
    if (layout && !a->group_boxes.ptr && a->n_strands > 0) {
        const size_t groups = (size_t(a->n_strands) + 7) / 8;
        if (a->ctx->alloc(a->group_boxes, groups * 2 * sizeof(int4)) != RVH_OK) set_error("");
    }
    if (layout && a->group_boxes.ptr) {
        view->group_box = static_cast<int4*>(a->group_boxes.ptr);
        view->box_tag_read = (a->pending && a->box_layout == layout) ? a->box_tag : 0u;
        gu->box_tag = a->box_tag + 1u ? a->box_tag + 1u : 1u;
        view->box_tag_write = gu->box_tag;
    }
}

// group_pending (an owner of a grid group): whether any asset of the group has friction
// pending in grid[pend]; -1 uses the asset's own state.
rvh_status prepare_asset(Asset* a, int mode, const rvh_frame& f, cudaStream_t s, DevAsset* view, GridUse* gu,
                         uint32_t layout, int group_pending = -1) {
    *gu = GridUse{};
    if (!a->params.grid_enabled) {
        *view = a->device_view(f, -1);
        return RVH_OK;
    }
    if (!a->grid[0].ptr || !a->grid[1].ptr || !a->grid[2].ptr)
        return fail(RVH_ERR_STATE, "batch: an asset's grids are held by a request server");
    if (mode == MODE_FINISH) {
        rvh_frame fp = f;
        fp.dt = a->dt_prev;
        *view = a->device_view(fp, a->pend);
        gu->prev = a->pend;
        return RVH_OK;
    }
    const bool held = group_pending < 0 ? a->pending : group_pending != 0;   // grid[pend] still needed
    gu->prev = held ? a->pend : -1;
    gu->t = a->pick_grid(gu->prev, -1);
    if (a->grid_dirty[gu->t]) RVH_CUDA(cudaMemsetAsync(a->grid[gu->t].ptr, 0, a->grid_bytes(), s));
    gu->u = a->pick_grid(gu->prev, gu->t);
    *view = a->device_view(f, gu->t, a->pending ? gu->prev : -1, gu->u);
    attach_group_boxes(a, view, gu, layout);
    return RVH_OK;
}

// A grid group's member: the owner's choice of grids (og), its own pending friction.
rvh_status prepare_member(Asset* a, const GridUse& og, const rvh_frame& f, DevAsset* view, GridUse* gu,
                          uint32_t layout) {
    *gu = og;
    gu->box_tag = 0;
    if (a->pending && a->pend != og.prev) return fail(RVH_ERR_STATE, "batch: a grid group's pending grids disagree");
    *view = a->device_view(f, og.t, a->pending ? og.prev : -1, og.u);
    attach_group_boxes(a, view, gu, layout);
    return RVH_OK;
}

void commit_asset(Asset* a, int mode, const GridUse& gu, float dt, uint32_t layout, bool member = false) {
    if (!a->params.grid_enabled) return;
    if (member && mode != MODE_FINISH) {   // the owner's commit keeps the group's grid flags
        a->last_grid = gu.t;
        a->pending = mode == MODE_FUSED;
        a->pend = gu.t;
        a->dt_prev = dt;
        a->box_tag = gu.box_tag ? gu.box_tag : a->box_tag;
        a->box_layout = gu.box_tag ? layout : 0u;
        return;
    }
    if (mode == MODE_FINISH) {
        a->pending = false;
        a->grid_dirty[gu.prev] = true;
        return;
    }
    if (gu.prev >= 0) a->grid_dirty[gu.prev] = true;
    a->grid_dirty[gu.u] = false;  // the launch's clear items zero it
    a->grid_dirty[gu.t] = true;
    a->last_grid = gu.t;
    a->pending = mode == MODE_FUSED;
    a->pend = gu.t;
    a->dt_prev = dt;
    a->box_tag = gu.box_tag ? gu.box_tag : a->box_tag;
    a->box_layout = gu.box_tag ? layout : 0u;
}

void destroy(Batch* b) {
    if (!b) return;
    if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
    if (b->copy_stream) cudaStreamSynchronize(b->copy_stream), cudaStreamDestroy(b->copy_stream);
    for (int i = 0; i < 2; ++i) {
        if (b->packed[i]) cudaEventDestroy(b->packed[i]);
        if (b->copied[i]) cudaEventDestroy(b->copied[i]);
        if (b->ctx) b->ctx->free(b->pos_stage[i]);
    }
    if (b->ctx) b->ctx->free(b->d_first);
    for (auto& e : b->ev_pairs) cudaEventDestroy(e.first), cudaEventDestroy(e.second);
    for (auto& e : b->ev_free) cudaEventDestroy(e.first), cudaEventDestroy(e.second);
    if (b->finisher) dyn_batch_free(b->finisher);
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
    b.min_tile_points = kMinTilePoints;   // launches of any size keep one grouping per asset
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
                            const std::vector<int>& modes, cudaStream_t s, cudaEvent_t ev_start, cudaEvent_t ev_stop,
                            int64_t* points) {
    Batch& b = d->b;
    b.assets = assets;
    b.modes = modes;
    b.entry_step.clear();
    // a launch carries what the requests of the moment need: tiles sized so every CTA
    // gets about sixteen (small launches would otherwise leave most CTAs idle, and a
    // few large tiles leave a tail; at 16 requests per launch 16 per CTA served
    // 3 % more point-steps than 8, 14 % more than 4 and 53 % more than 2)
    int64_t launch_pts = 0;
    for (Asset* a : assets) launch_pts += int64_t(a->n_strands) * a->n_points;
    const int64_t per_tile = launch_pts / std::max<int64_t>(1, 16 * int64_t(b.n_ctas));
    plan(b, 0, int(std::min<int64_t>(kTargetPointsA, std::max<int64_t>(kMinTilePoints, per_tile))));
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
    std::vector<GridUse> gus(assets.size());
    for (size_t i = 0; i < assets.size(); ++i) {
        rvh_status ps = prepare_asset(assets[i], modes[i], frames[i], s, &b.h_stage[slot][i], &gus[i],
                                      box_layout_of(b, i));
        if (ps != RVH_OK) return ps;
        b.h_stage[slot][i].group_rounds = b.group_rounds[i];
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
    for (size_t i = 0; i < assets.size(); ++i)
        commit_asset(assets[i], modes[i], gus[i], frames[i].dt, box_layout_of(b, i));
    return RVH_OK;
}

// Several fused steps of each asset in ONE persistent launch: the entries of an
// asset's step s + 1 wait (on the device, bounded) for every phase-A item and
// clear of its step s, whose positions they read, whose splat grid they gather
// from and whose cleared grid they splat into.  The three grids rotate from
// step to step: (pending, target, to clear) -> (target, to clear, pending).
// modes: MODE_FUSED (steps[i] >= 1) or MODE_FINISH (steps[i] == 1); frames:
// per asset, its steps' frames in order.
rvh_status dyn_batch_launch_steps(DynBatch* d, const std::vector<Asset*>& assets, const std::vector<int>& steps,
                                  const std::vector<int>& modes, const std::vector<rvh_frame>& frames, cudaStream_t s,
                                  cudaEvent_t ev_start, cudaEvent_t ev_stop) {
    Batch& b = d->b;
    const size_t na = assets.size();
    std::vector<size_t> first(na), first_frame(na);
    std::vector<Asset*> ents;
    std::vector<int> emode, estep;
    size_t nf = 0;
    for (size_t i = 0; i < na; ++i) {
        if (steps[i] < 1 || (modes[i] != MODE_FUSED && (modes[i] != MODE_FINISH || steps[i] != 1)))
            return fail(RVH_ERR_INVALID_ARG, "server launch: bad steps or mode");
        first[i] = ents.size();
        first_frame[i] = nf;
        nf += size_t(steps[i]);
        for (int k = 0; k < steps[i]; ++k) {
            ents.push_back(assets[i]);
            emode.push_back(modes[i]);
            estep.push_back(k);
        }
    }
    if (frames.size() != nf) return fail(RVH_ERR_INVALID_ARG, "server launch: one frame per step");
    b.assets = ents;
    b.modes = emode;
    b.entry_step = estep;
    int64_t launch_pts = 0;
    for (Asset* a : ents) launch_pts += int64_t(a->n_strands) * a->n_points;
    const int64_t per_tile = launch_pts / std::max<int64_t>(1, 16 * int64_t(b.n_ctas));
    plan(b, 0, int(std::min<int64_t>(kTargetPointsA, std::max<int64_t>(kMinTilePoints, per_tile))));
    b.dev.n_items = int32_t(b.items.size());
    if (b.items.empty()) return RVH_OK;
    rvh_status st = dyn_reserve(d, ents.size(), b.items.size());
    if (st != RVH_OK) return st;
    const int slot = b.slot;
    b.slot ^= 1;
    RVH_CUDA(cudaEventSynchronize(b.staged[slot]));
    DevAsset* stage = b.h_stage[slot];
    struct After {   // what each asset's state becomes once the launch is enqueued
        GridUse gu;
        int t = -1, u = -1, third = -1;
        bool third_dirty = false;
        uint32_t tag = 0;
        float dt = 0.f;
    };
    std::vector<After> after(na);
    for (size_t i = 0; i < na; ++i) {
        Asset* a = assets[i];
        const size_t e0 = first[i];
        const rvh_frame* fr = frames.data() + first_frame[i];
        const uint32_t layout = box_layout_of(b, e0);
        After& af = after[i];
        af.dt = fr[steps[i] - 1].dt;
        if (modes[i] == MODE_FINISH || !a->params.grid_enabled) {
            if (modes[i] == MODE_FINISH) {
                rvh_status ps = prepare_asset(a, MODE_FINISH, fr[0], s, &stage[e0], &af.gu, layout);
                if (ps != RVH_OK) return ps;
            } else {
                for (int k = 0; k < steps[i]; ++k) {
                    stage[e0 + k] = a->device_view(fr[k], -1);
                    stage[e0 + k].wait_entry = k > 0 ? int32_t(e0 + k - 1) : -1;
                }
            }
        } else {
            if (!a->grid[0].ptr || !a->grid[1].ptr || !a->grid[2].ptr)
                return fail(RVH_ERR_STATE, "server launch: an asset has no grids");
            int prev = a->pending ? a->pend : -1;
            int t = a->pick_grid(prev, -1);
            if (a->grid_dirty[t]) RVH_CUDA(cudaMemsetAsync(a->grid[t].ptr, 0, a->grid_bytes(), s));
            int u = a->pick_grid(prev, t);
            af.third_dirty = steps[i] > 1 || prev >= 0;
            if (layout && !a->group_boxes.ptr && a->n_strands > 0) {
                const size_t groups = (size_t(a->n_strands) + 7) / 8;
                if (a->ctx->alloc(a->group_boxes, groups * 2 * sizeof(int4)) != RVH_OK) set_error("");
            }
            const bool tags = layout && a->group_boxes.ptr;
            uint32_t tag = a->box_tag;
            for (int k = 0; k < steps[i]; ++k) {
                const int gather = k == 0 ? (a->pending ? prev : -1) : prev;
                DevAsset& v = stage[e0 + k];
                v = a->device_view(fr[k], t, gather, u);
                if (k > 0) v.dt_prev = fr[k - 1].dt;
                v.wait_entry = k > 0 ? int32_t(e0 + k - 1) : -1;
                if (tags) {
                    v.group_box = static_cast<int4*>(a->group_boxes.ptr);
                    v.box_tag_read = k > 0 ? tag : ((a->pending && a->box_layout == layout) ? a->box_tag : 0u);
                    tag = tag + 1u ? tag + 1u : 1u;
                    v.box_tag_write = tag;
                }
                const int third = 3 - t - u;   // (gathered, target, cleared) -> (target, cleared, gathered)
                if (k + 1 < steps[i]) {
                    prev = t;
                    t = u;
                    u = third;
                } else {
                    af.t = t;
                    af.u = u;
                    af.third = third;
                }
            }
            af.tag = tags ? tag : 0u;
        }
        for (int k = 0; k < steps[i]; ++k) stage[e0 + k].group_rounds = b.group_rounds[e0 + k];
    }
    for (size_t e = 0; e < ents.size(); ++e) d->h_need[slot][e] = b.need_a[e];
    std::memcpy(d->h_items[slot], b.items.data(), sizeof(WorkItem) * b.items.size());
    RVH_CUDA(cudaMemcpyAsync(b.d_assets.ptr, stage, sizeof(DevAsset) * ents.size(), cudaMemcpyHostToDevice, s));
    RVH_CUDA(cudaMemcpyAsync(b.d_items.ptr, d->h_items[slot], sizeof(WorkItem) * b.items.size(), cudaMemcpyHostToDevice, s));
    RVH_CUDA(cudaMemcpyAsync(b.d_need.ptr, d->h_need[slot], sizeof(unsigned) * ents.size(), cudaMemcpyHostToDevice, s));
    RVH_CUDA(cudaEventRecord(b.staged[slot], s));
    if (ev_start) RVH_CUDA(cudaEventRecord(ev_start, s));
    rvh_status ls = enqueue_launch(&b, s);
    if (ls != RVH_OK) return ls;
    if (ev_stop) RVH_CUDA(cudaEventRecord(ev_stop, s));
    for (size_t i = 0; i < na; ++i) {
        Asset* a = assets[i];
        const After& af = after[i];
        if (modes[i] == MODE_FINISH) {
            commit_asset(a, MODE_FINISH, af.gu, af.dt, 0u);
            continue;
        }
        if (!a->params.grid_enabled) continue;
        a->grid_dirty[af.t] = true;
        a->grid_dirty[af.u] = false;   // the last step's clear items zero it
        if (af.third_dirty) a->grid_dirty[af.third] = true;
        a->last_grid = af.t;
        a->pending = true;
        a->pend = af.t;
        a->dt_prev = af.dt;
        a->box_tag = af.tag ? af.tag : a->box_tag;
        a->box_layout = af.tag ? box_layout_of(b, first[i]) : 0u;
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
            lanes = 8;   // the tuner's pick on the 256-head workload (4 lanes: 7.3-7.5 ms a step against 5.4 ms)
        }
        set_error(keep);
    }
    if (!batch_supported(lanes)) return fail(RVH_ERR_UNSUPPORTED, "batch: lanes_per_strand must be 1, 4, 8, 16 or 32");
    RVH_DEVICE(ctx->device);
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
        b->modes.push_back(d.full_steps ? MODE_FULL : MODE_FUSED);
        b->first_point.push_back(b->n_points);
        b->n_points += int64_t(assets[i]->n_strands) * assets[i]->n_points;
    }
    // grid groups: every asset of a group in the batch, fused steps only (a full step's gather
    // would wait for the phase A of every member, not of its own asset)
    b->grid_root.assign(b->assets.size(), -1);
    for (size_t i = 0; i < b->assets.size(); ++i) {
        const Asset* a = b->assets[i];
        if (!a->grid_grouped() || !a->params.grid_enabled) continue;
        const Asset* owner = a->grid_owner ? a->grid_owner : a;
        size_t members_here = 0;
        int root = -1;
        for (size_t j = 0; j < b->assets.size(); ++j) {
            if (b->assets[j] == owner) root = int(j);
            if (b->assets[j]->grid_owner == owner) ++members_here;
        }
        if (root < 0 || members_here != owner->grid_members.size()) {
            destroy(b);
            return fail(RVH_ERR_INVALID_ARG, "batch_create: a grid group's assets must all be in the batch");
        }
        if (d.full_steps) {
            destroy(b);
            return fail(RVH_ERR_UNSUPPORTED, "batch_create: assets sharing a grid take fused steps only");
        }
        b->grid_root[i] = root;
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
    // phase-A items of about 4,096 points, smaller when the batch holds too few points to give
    // every CTA about eight (one large asset alone would otherwise leave a long tail)
    int64_t batch_pts = 0;
    for (const Asset* a : b->assets) batch_pts += int64_t(a->n_strands) * a->n_points;
    const int64_t per_tile = batch_pts / std::max<int64_t>(1, 8 * int64_t(b->n_ctas));
    plan(*b, d.strands_per_tile, int(std::min<int64_t>(kTargetPointsA, std::max<int64_t>(kMinTilePoints, per_tile))));
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
    if (!b) return RVH_OK;
    DeviceGuard g(b->ctx ? b->ctx->device : 0);   // releases even if the switch fails
    destroy(b);
    return RVH_OK;
}

}  // extern "C"

namespace rvh {
namespace {

// One batched step; with xyz set, every point's new position is also written
// there (asset after asset, xyz per point) by the step itself.
rvh_status batch_step(rvh_batch* b, const rvh_frame* frames, cudaStream_t s, float* xyz) {
    if (!b || (!frames && !b->assets.empty())) return fail(RVH_ERR_INVALID_ARG, "batch_step: NULL argument");
    for (size_t i = 0; i < b->assets.size(); ++i) {
        const rvh_status vs = validate_frame(frames[i]);
        if (vs != RVH_OK) return vs;
    }
    if (b->items.empty()) return RVH_OK;
    RVH_DEVICE(b->ctx->device);
    const int slot = b->slot;
    b->slot ^= 1;
    RVH_CUDA(cudaEventSynchronize(b->staged[slot]));  // the copy that last read this staging buffer is done
    DevAsset* st = b->h_stage[slot];
    std::vector<GridUse> gus(b->assets.size());
    const size_t na = b->assets.size();
    // owners and assets with grids of their own first, then the members of grid groups
    for (int pass = 0; pass < 2; ++pass)
        for (size_t i = 0; i < na; ++i) {
            const int root = b->grid_root.empty() ? -1 : b->grid_root[i];
            const bool member = root >= 0 && root != int(i);
            if (member != (pass == 1)) continue;
            rvh_status ps;
            if (member) {
                ps = prepare_member(b->assets[i], gus[root], frames[i], &st[i], &gus[i], box_layout_of(*b, i));
            } else {
                int group_pending = -1;
                if (root == int(i)) {
                    const Asset* o = b->assets[i];
                    group_pending = o->pending ? 1 : 0;
                    for (const Asset* m : o->grid_members) group_pending |= m->pending ? 1 : 0;
                }
                ps = prepare_asset(b->assets[i], b->modes[i], frames[i], s, &st[i], &gus[i], box_layout_of(*b, i),
                                   group_pending);
            }
            if (ps != RVH_OK) return ps;
            st[i].group_rounds = b->group_rounds[i];
            st[i].pos_xyz = xyz ? xyz + 3 * b->first_point[i] : nullptr;
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
    for (size_t i = 0; i < na; ++i) {
        const int root = b->grid_root.empty() ? -1 : b->grid_root[i];
        commit_asset(b->assets[i], b->modes[i], gus[i], frames[i].dt, box_layout_of(*b, i), root >= 0 && root != int(i));
    }
    return RVH_OK;
}

}  // namespace
}  // namespace rvh

extern "C" {

rvh_status rvh_batch_step(rvh_batch* b, const rvh_frame* frames, void* stream) {
    TraceRange trace("rvh_batch_step");
    if (!b) return fail(RVH_ERR_INVALID_ARG, "batch_step: NULL argument");
    return batch_step(b, frames, stream ? static_cast<cudaStream_t>(stream) : b->ctx->stream, nullptr);
}

// Every pending asset's loop 3 in ONE persistent launch of gather-only items
// (the server's finish mode): the same tile code as the per-asset finish, so
// the same bits, without a launch sequence per asset.
rvh_status rvh_batch_finish(rvh_batch* b, void* stream) {
    TraceRange trace("rvh_batch_finish");
    if (!b) return fail(RVH_ERR_INVALID_ARG, "batch_finish: NULL");
    RVH_DEVICE(b->ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->ctx->stream;
    std::vector<Asset*> pend;
    for (Asset* a : b->assets)
        if (a->pending) pend.push_back(a);
    if (pend.empty()) return RVH_OK;
    if (!b->finisher) {
        rvh_status st;
        b->finisher = dyn_batch_new(b->ctx, batch_supported(b->lanes) ? b->lanes : 8, &st);
        if (!b->finisher) return st;
    }
    std::vector<rvh_frame> frames(pend.size());   // finish mode takes each asset's own dt of that step
    for (size_t i = 0; i < pend.size(); ++i) frames[i].dt = pend[i]->dt_prev;
    const std::vector<int> modes(pend.size(), MODE_FINISH);
    rvh_status st = dyn_batch_launch(b->finisher, pend, frames, modes, s, nullptr, nullptr, nullptr);
    if (st != RVH_OK) return st;
    return RVH_OK;
}

rvh_status rvh_batch_check(rvh_batch* b) {
    if (!b) return fail(RVH_ERR_INVALID_ARG, "batch_check: NULL");
    RVH_DEVICE(b->ctx->device);
    RVH_CUDA(cudaStreamSynchronize(b->ctx->stream));
    RVH_CUDA(cudaDeviceSynchronize());
    int err = 0;
    RVH_CUDA(cudaMemcpy(&err, b->d_error.ptr, sizeof(int), cudaMemcpyDeviceToHost));
    if (err != 0) {
        RVH_CUDA(cudaMemset(b->d_error.ptr, 0, sizeof(int)));
        return fail(err, "batch: a phase-B tile gave up waiting for its asset's phase A");
    }
    if (b->finisher) return dyn_batch_check(b->finisher);
    return RVH_OK;
}

}  // extern "C"

namespace rvh {
namespace {

// First use of a batch's position read-back: two staging slots, the pack
// kernel's chunk table, the copy stream and its events.
rvh_status ensure_staging(rvh_batch* b) {
    if (b->copy_stream) return RVH_OK;
    const size_t n4 = size_t(b->n_points) * 16u;
    rvh_status st;
    for (int i = 0; i < 2; ++i)
        if ((st = b->ctx->alloc(b->pos_stage[i], n4)) != RVH_OK) return st;
    std::vector<PackChunk> chunks;
    long long acc = 0;
    for (size_t a = 0; a < b->assets.size(); ++a) {
        const int ns = b->assets[a]->n_strands, n = b->assets[a]->n_points;
        const int per = std::max(1, 8192 / n);   // strands per chunk
        for (int s0 = 0; s0 < ns; s0 += per) {
            const int cnt = std::min(per, ns - s0);
            chunks.push_back(PackChunk{int(a), s0, cnt, n, acc});
            acc += (long long)cnt * n;
        }
    }
    b->n_pack_chunks = int(chunks.size());
    if ((st = b->ctx->alloc(b->d_first, sizeof(PackChunk) * std::max<size_t>(1, chunks.size()))) != RVH_OK) return st;
    if (!chunks.empty())
        RVH_CUDA(cudaMemcpy(b->d_first.ptr, chunks.data(), sizeof(PackChunk) * chunks.size(), cudaMemcpyHostToDevice));
    RVH_CUDA(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        RVH_CUDA(cudaEventCreateWithFlags(&b->packed[i], cudaEventDisableTiming));
        RVH_CUDA(cudaEventCreateWithFlags(&b->copied[i], cudaEventDisableTiming));
    }
    return RVH_OK;
}

// The staged positions of `slot` are complete on stream s: copy them to the
// host on the copy stream.
rvh_status copy_out(rvh_batch* b, int slot, cudaStream_t s, void* host_dst, size_t bytes) {
    RVH_CUDA(cudaEventRecord(b->packed[slot], s));
    RVH_CUDA(cudaStreamWaitEvent(b->copy_stream, b->packed[slot], 0));
    RVH_CUDA(cudaMemcpyAsync(host_dst, b->pos_stage[slot].ptr, bytes, cudaMemcpyDeviceToHost, b->copy_stream));
    RVH_CUDA(cudaEventRecord(b->copied[slot], b->copy_stream));
    return RVH_OK;
}

}  // namespace
}  // namespace rvh

extern "C" {

rvh_status rvh_batch_read_positions_async(rvh_batch* b, void* host_dst, size_t bytes, void* stream) {
    if (!b || (!host_dst && bytes)) return fail(RVH_ERR_INVALID_ARG, "batch_read_positions: NULL argument");
    const size_t n4 = size_t(b->n_points) * 16u, n3 = size_t(b->n_points) * 12u;
    if (bytes != n4 && bytes != n3)
        return fail(RVH_ERR_INVALID_ARG, "batch_read_positions: size must be 16 (float4) or 12 (xyz) * total points");
    if (!bytes) return RVH_OK;
    const bool xyz = bytes == n3 && n3 != n4;
    RVH_DEVICE(b->ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->ctx->stream;
    rvh_status st = ensure_staging(b);
    if (st != RVH_OK) return st;
    const int slot = b->pos_slot;
    b->pos_slot ^= 1;
    RVH_CUDA(cudaStreamWaitEvent(s, b->copied[slot], 0));   // the copy that last read this slot is done
    const int blocks = std::max(1, std::min(b->n_pack_chunks, b->ctx->sm_count * 8));
    const DevAsset* assets = static_cast<const DevAsset*>(b->d_assets.ptr);
    const PackChunk* chunks = static_cast<const PackChunk*>(b->d_first.ptr);
    int nc = b->n_pack_chunks;
    void* out = b->pos_stage[slot].ptr;
    void* args[] = {&assets, &chunks, &nc, &out};
    const void* fn = xyz ? reinterpret_cast<const void*>(&k_pack_positions<true>)
                         : reinterpret_cast<const void*>(&k_pack_positions<false>);
    RVH_CUDA(cudaLaunchKernel(fn, dim3(unsigned(blocks)), dim3(kThreads), args, 0, s));
    return copy_out(b, slot, s, host_dst, bytes);
}

rvh_status rvh_batch_step_read_positions(rvh_batch* b, const rvh_frame* frames, void* host_dst, size_t bytes,
                                         void* stream) {
    TraceRange trace("rvh_batch_step_read_positions");
    if (!b || (!host_dst && bytes)) return fail(RVH_ERR_INVALID_ARG, "batch_step_read_positions: NULL argument");
    if (bytes != size_t(b->n_points) * 12u)
        return fail(RVH_ERR_INVALID_ARG, "batch_step_read_positions: size must be 12 (xyz) * total points");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->ctx->stream;
    if (!bytes) return batch_step(b, frames, s, nullptr);
    RVH_DEVICE(b->ctx->device);
    rvh_status st = ensure_staging(b);
    if (st != RVH_OK) return st;
    const int slot = b->pos_slot;
    b->pos_slot ^= 1;
    RVH_CUDA(cudaStreamWaitEvent(s, b->copied[slot], 0));   // the copy that last read this slot is done
    if ((st = batch_step(b, frames, s, static_cast<float*>(b->pos_stage[slot].ptr))) != RVH_OK) return st;
    return copy_out(b, slot, s, host_dst, bytes);
}

rvh_status rvh_batch_positions_wait(rvh_batch* b) {
    if (!b) return fail(RVH_ERR_INVALID_ARG, "batch_positions_wait: NULL");
    if (!b->copy_stream) return RVH_OK;
    RVH_DEVICE(b->ctx->device);
    RVH_CUDA(cudaStreamSynchronize(b->copy_stream));
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
    RVH_DEVICE(b->ctx->device);
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
