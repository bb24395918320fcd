// rvh_tuner.cpp — autotuner for the batched step.
//
// Candidates: lanes per strand {1, 4, 8, 16, 32} (strands per warp 32, 8, 4, 2, 1),
// phase-A tile size {1, 2, 4} rounds of kWarps * strands-per-warp strands,
// and optionally the grid resolution of every grid-enabled asset (same
// bounds, finer or coarser cells).  Each candidate times real batched steps
// of the caller's assets with CUDA events; the strand records are snapshotted
// before and restored after every trial, so tuning does not advance the
// simulation.  Results are cached per workload signature in the context.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rvh_internal.hpp"

namespace rvh {

namespace {

std::mutex g_cache_mu;
std::map<std::string, rvh_tune_result> g_cache;

// (n_points, log2 strand bucket, grid cells) per asset, sorted: assets of
// similar shape share tuned settings.
std::string signature(rvh_asset* const* assets, int n) {
    std::vector<std::string> parts;
    for (int i = 0; i < n; ++i) {
        const Asset* a = assets[i];
        int b = 0;
        while ((1 << (b + 1)) <= std::max(1, a->n_strands)) ++b;
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%d:%d:%zu", a->n_points, b,
                      a->params.grid_enabled ? size_t(a->params.grid_dims[0]) * a->params.grid_dims[1] *
                                                   a->params.grid_dims[2]
                                             : size_t(0));
        parts.push_back(buf);
    }
    std::sort(parts.begin(), parts.end());
    std::string s;
    for (auto& p : parts) s += p + ",";
    return s;
}

rvh_status set_grid_res(Asset* a, int res, const rvh_sim_params& orig) {
    rvh_sim_params p = orig;
    if (!p.grid_enabled || res <= 0) return rvh_asset_set_params(static_cast<rvh_asset*>(a), &orig);
    const float ext = orig.grid_h * float(orig.grid_dims[0]);
    p.grid_dims[0] = p.grid_dims[1] = p.grid_dims[2] = res;
    p.grid_h = ext / float(res);
    return rvh_asset_set_params(static_cast<rvh_asset*>(a), &p);
}

}  // namespace
}  // namespace rvh

using namespace rvh;

extern "C" {

rvh_status rvh_tune_batch(rvh_context* ctx, rvh_asset* const* assets, int32_t n, const rvh_frame* frames,
                          const rvh_tune_desc* desc, rvh_tune_result* out) {
    if (!ctx || !assets || n < 1 || !frames || !out) return fail(RVH_ERR_INVALID_ARG, "tune_batch: bad argument");
    rvh_tune_desc d{};
    d.steps = 3;
    if (desc) d = *desc;
    if (d.steps < 1) d.steps = 3;
    if (d.n_grid_res < 0 || d.n_grid_res > 8) return fail(RVH_ERR_INVALID_ARG, "tune_batch: at most 8 grid sizes");
    const std::string key = signature(assets, n) + (d.tune_grid ? "|grid" : "");
    if (d.use_cache) {
        std::lock_guard<std::mutex> g(g_cache_mu);
        auto it = g_cache.find(key);
        if (it != g_cache.end()) {
            *out = it->second;
            return RVH_OK;
        }
    }
    RVH_DEVICE(ctx->device);
    // pending friction first, so that the snapshot is a finished state
    for (int i = 0; i < n; ++i) {
        rvh_status fs = finish_pending(assets[i], ctx->stream);
        if (fs != RVH_OK) return fs;
    }
    RVH_CUDA(cudaDeviceSynchronize());
    // snapshot the records of every asset
    std::vector<DevBuf> snap(n);
    std::vector<rvh_sim_params> orig(n);
    auto release = [&]() {
        for (auto& b : snap) ctx->free(b);
    };
    for (int i = 0; i < n; ++i) {
        orig[i] = assets[i]->params;
        rvh_status s = ctx->alloc(snap[i], assets[i]->record_bytes());
        if (s != RVH_OK) {
            release();
            return s;
        }
        if (assets[i]->record_bytes())
            RVH_CUDA(cudaMemcpy(snap[i].ptr, assets[i]->strands.ptr, assets[i]->record_bytes(), cudaMemcpyDeviceToDevice));
    }
    // the snapshot back, with no pending friction, no stored group boxes and grids to be
    // cleared before their next use (a trial's grids and boxes describe its own last step)
    auto restore = [&]() -> rvh_status {
        RVH_CUDA(cudaDeviceSynchronize());
        for (int i = 0; i < n; ++i) {
            Asset* a = assets[i];
            if (a->record_bytes())
                RVH_CUDA(cudaMemcpy(a->strands.ptr, snap[i].ptr, a->record_bytes(), cudaMemcpyDeviceToDevice));
            a->pending = false;
            a->box_layout = 0u;
            a->last_grid = -1;
            for (int g = 0; g < 3; ++g) a->grid_dirty[g] = true;
        }
        return RVH_OK;
    };
    std::vector<int> res_list = {0};
    if (d.tune_grid && d.n_grid_res > 0) res_list.assign(d.grid_res, d.grid_res + d.n_grid_res);
    rvh_tune_result r{};
    r.best_ms = 1e30f;
    const int lanes_c[5] = {1, 4, 8, 16, 32};
    const int tile_c[4] = {0, 1, 2, 4};   // rounds per phase-A item; 0: whole groups near 4,096 points
    rvh_status st = RVH_OK;
    for (int res : res_list) {
        for (int i = 0; i < n && st == RVH_OK; ++i) st = set_grid_res(assets[i], res, orig[i]);
        for (int li = 0; li < 5 && st == RVH_OK; ++li)
            for (int ti = 0; ti < 4 && st == RVH_OK; ++ti) {
                const int lanes = lanes_c[li];
                const int tile = tile_c[ti] * kWarps * (32 / lanes);
                rvh_batch_desc bd{lanes, tile, 0, 1, 0, 0};
                rvh_batch* b = nullptr;
                st = rvh_batch_create(ctx, assets, n, &bd, &b);
                if (st != RVH_OK) break;
                rvh_batch_step(b, frames, nullptr);  // warm-up
                rvh_batch_timing_enable(b, 1);
                for (int k = 0; k < d.steps && st == RVH_OK; ++k) st = rvh_batch_step(b, frames, nullptr);
                double ms = 0.0;
                int32_t cnt = 0;
                if (st == RVH_OK) st = rvh_batch_timing_read(b, &ms, &cnt);
                if (st == RVH_OK) st = rvh_batch_check(b);
                rvh_batch_destroy(b);
                if (st == RVH_OK) st = restore();
                if (st != RVH_OK) break;
                const float per = float(ms / std::max(1, int(cnt)));
                if (r.n_tried < 96) {
                    r.tried_lanes[r.n_tried] = lanes;
                    r.tried_tile[r.n_tried] = tile;
                    r.tried_res[r.n_tried] = res;
                    r.tried_ms[r.n_tried] = per;
                    r.n_tried++;
                }
                if (per < r.best_ms) {
                    r.best_ms = per;
                    r.lanes_per_strand = lanes;
                    r.strands_per_tile = tile;
                    r.grid_res = res;
                }
            }
    }
    // leave the assets with the chosen grid size (or their own when the grid was not tuned)
    for (int i = 0; i < n; ++i) {
        rvh_status s2 = set_grid_res(assets[i], d.tune_grid ? r.grid_res : 0, orig[i]);
        if (st == RVH_OK) st = s2;
    }
    if (st == RVH_OK) st = restore();
    release();
    if (st != RVH_OK) return st;
    *out = r;
    std::lock_guard<std::mutex> g(g_cache_mu);
    g_cache[key] = r;
    return RVH_OK;
}

rvh_status rvh_tune_lookup(rvh_asset* const* assets, int32_t n, int32_t tuned_grid, rvh_tune_result* out) {
    if (!assets || n < 1 || !out) return fail(RVH_ERR_INVALID_ARG, "tune_lookup: bad argument");
    const std::string key = signature(assets, n) + (tuned_grid ? "|grid" : "");
    std::lock_guard<std::mutex> g(g_cache_mu);
    auto it = g_cache.find(key);
    if (it == g_cache.end()) return fail(RVH_ERR_STATE, "tune_lookup: no tuned result for this workload");
    *out = it->second;
    return RVH_OK;
}

}  // extern "C"
