// rvh_server.cpp — a request loop with continuous batching for resident
// characters (the serving counterpart of the reference's per-frame
// UpdateTime -> Frame -> translateSphere loop, src/main.cpp:257-285).
//
// Every character's Strand records stay in HBM.  A request asks for k steps of
// one character.  Each launch advances every ADMITTED request by up to
// steps_per_launch steps in one persistent batch launch; a request holds its
// slot from admission until its last step is enqueued (so a launch carries at
// most max_active requests), its character until that step completes.
// Requests are admitted in arrival order as soon as (a) a slot is free, (b) its
// character has no other request in flight, and (c) the character's grid
// scratch fits the server's HBM budget (or the character still holds its grids).
// Up to `pipeline_depth` launches are in flight, so new arrivals join the next
// launch while earlier ones still run on the device.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <new>
#include <thread>
#include <vector>

#include "../../include/rvh_scene.h"
#include "rvh_internal.hpp"

namespace rvh {

namespace {

// First-fit allocator over one device slab (offsets in bytes, 256-B aligned).
class SlabPool {
public:
    void init(size_t bytes) {
        free_.clear();
        if (bytes) free_[0] = bytes;
        size_ = bytes;
    }
    bool take(size_t bytes, size_t* off) {
        bytes = (bytes + 255) & ~size_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes;
                const size_t noff = it->first + bytes;
                free_.erase(it);
                if (rest) free_[noff] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void give(size_t off, size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }

private:
    std::map<size_t, size_t> free_;
    size_t size_ = 0, used_ = 0;
};

struct Character {
    Asset* asset = nullptr;
    rvh_wind_desc wind{};
    bool has_wind = false;
    float dt = 1.0f / 60.0f;
    int64_t steps = 0;      // steps completed or enqueued so far
    bool busy = false;
    // grid scratch lent from the pool; held after a request while the last fused step's
    // friction is pending, until a later request continues it or the pool needs the space
    bool held = false;
    bool finishing = false; // a launch in flight applies the pending friction, then releases
    size_t off = 0, bytes = 0;
    int64_t last_launch = 0;
};

struct Active {
    int req;
    int remaining;          // steps still to enqueue
    int in_flight = 0;      // launches containing this request not yet completed
};

struct Launch {
    cudaEvent_t start, stop;
    std::vector<int> reqs;  // requests with steps in this launch
    std::vector<int> nsteps;   // how many of each
    std::vector<int> last;  // requests whose final step is in this launch
    std::vector<int> finish;   // characters whose pending friction this launch applies
    int64_t points = 0;
};

double pct(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double idx = p * double(v.size() - 1);
    const size_t lo = size_t(std::floor(idx)), hi = std::min(v.size() - 1, lo + 1);
    return v[lo] + (v[hi] - v[lo]) * (idx - double(lo));
}

}  // namespace

struct Server {
    Context* ctx = nullptr;
    rvh_server_desc desc{};
    std::vector<Character> chars;
    DynBatch* batch = nullptr;
    DevBuf slab;
    SlabPool pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;
};

}  // namespace rvh

struct rvh_server : rvh::Server {};

using namespace rvh;

extern "C" {

rvh_status rvh_server_create(rvh_context* ctx, const rvh_server_desc* desc, rvh_server** out) {
    if (!ctx || !out) return fail(RVH_ERR_INVALID_ARG, "server_create: NULL argument");
    *out = nullptr;
    rvh_server_desc d{};
    d.max_active = 16;
    d.lanes_per_strand = 8;
    d.pipeline_depth = 2;
    if (desc) d = *desc;
    if (d.max_active < 1 || d.max_active > 4096) return fail(RVH_ERR_INVALID_ARG, "server: max_active in [1, 4096]");
    if (d.pipeline_depth < 1 || d.pipeline_depth > 8) return fail(RVH_ERR_INVALID_ARG, "server: pipeline_depth in [1, 8]");
    if (d.steps_per_launch == 0) d.steps_per_launch = 1;
    if (d.steps_per_launch < 1 || d.steps_per_launch > 16)
        return fail(RVH_ERR_INVALID_ARG, "server: steps_per_launch in [1, 16]");
    if (!d.lanes_per_strand) d.lanes_per_strand = 8;
    RVH_DEVICE(ctx->device);
    rvh_server* s = new (std::nothrow) rvh_server();
    if (!s) return fail(RVH_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->ctx = ctx;
    s->desc = d;
    rvh_status st;
    s->batch = dyn_batch_new(ctx, d.lanes_per_strand, &st);
    if (!s->batch) {
        delete s;
        return st;
    }
    if (d.scratch_budget_bytes) {
        if ((st = ctx->alloc(s->slab, d.scratch_budget_bytes)) != RVH_OK) {
            dyn_batch_free(s->batch);
            delete s;
            return st;
        }
        s->pool.init(s->slab.bytes);
    }
    *out = s;
    return RVH_OK;
}

rvh_status rvh_server_destroy(rvh_server* s) {
    if (!s) return RVH_OK;
    DeviceGuard g(s->ctx->device);   // releases even if the switch fails
    cudaStreamSynchronize(s->ctx->stream);
    for (auto& e : s->events) cudaEventDestroy(e.first), cudaEventDestroy(e.second);
    for (Character& c : s->chars) {
        Asset* a = c.asset;
        a->grid[0] = a->grid[1] = a->grid[2] = DevBuf{};
        a->pending = false;
        a->server_managed = false;
        ensure_grid(a);  // hand the asset back with grids of its own
    }
    dyn_batch_free(s->batch);
    s->ctx->free(s->slab);
    delete s;
    return RVH_OK;
}

rvh_status rvh_server_add_character(rvh_server* s, rvh_asset* a, const rvh_wind_desc* wind, float dt, int32_t* id) {
    if (!s || !a || !id) return fail(RVH_ERR_INVALID_ARG, "server_add_character: NULL argument");
    if (a->ctx != s->ctx) return fail(RVH_ERR_INVALID_ARG, "server_add_character: asset of another context");
    if (!std::isfinite(dt) || !(dt > 0.f)) return fail(RVH_ERR_INVALID_ARG, "server_add_character: dt must be > 0");
    for (const Character& c : s->chars)
        if (c.asset == a) return fail(RVH_ERR_INVALID_ARG, "server_add_character: asset already registered");
    if (a->params.grid_enabled && !s->slab.ptr)
        return fail(RVH_ERR_BUDGET, "server_add_character: the server has no scratch budget for grids");
    if (a->grid_grouped()) return fail(RVH_ERR_UNSUPPORTED, "server_add_character: the asset shares its grid");
    RVH_DEVICE(s->ctx->device);
    RVH_CUDA(cudaStreamSynchronize(s->ctx->stream));
    // the grids become per-request scratch lent from the server's pool
    rvh_status fs = finish_pending(a, s->ctx->stream);
    if (fs != RVH_OK) return fs;
    RVH_CUDA(cudaStreamSynchronize(s->ctx->stream));
    for (int g = 0; g < 3; ++g) s->ctx->free(a->grid[g]);
    a->server_managed = true;
    Character c;
    c.asset = a;
    c.dt = dt;
    if (wind) {
        c.wind = *wind;
        c.has_wind = true;
    }
    s->chars.push_back(c);
    *id = int32_t(s->chars.size() - 1);
    return RVH_OK;
}

rvh_status rvh_server_character_steps(rvh_server* s, int32_t id, int64_t* steps) {
    if (!s || !steps || id < 0 || id >= int32_t(s->chars.size()))
        return fail(RVH_ERR_INVALID_ARG, "server_character_steps: bad argument");
    *steps = s->chars[id].steps;
    return RVH_OK;
}

rvh_status rvh_server_run(rvh_server* s, const rvh_request* reqs, int32_t n, rvh_request_result* results,
                          rvh_server_stats* stats) {
    TraceRange trace("rvh_server_run");
    if (!s || (n > 0 && (!reqs || !results))) return fail(RVH_ERR_INVALID_ARG, "server_run: NULL argument");
    RVH_DEVICE(s->ctx->device);
    using clk = std::chrono::steady_clock;
    const cudaStream_t stream = s->ctx->stream;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return reqs[x].arrival_s < reqs[y].arrival_s; });
    for (int i = 0; i < n; ++i) {
        results[i] = rvh_request_result{};
        results[i].status = RVH_OK;
        if (reqs[i].character < 0 || reqs[i].character >= int32_t(s->chars.size()) || reqs[i].n_steps < 1) {
            results[i].status = RVH_ERR_INVALID_ARG;
        }
    }
    size_t next = 0;                      // next request (in arrival order) not yet queued
    std::deque<int> waiting;              // arrived, not admitted
    std::vector<Active> active;
    std::deque<Launch> flight;
    std::vector<cudaEvent_t> free_ev;
    auto get_ev = [&]() {
        if (!free_ev.empty()) {
            cudaEvent_t e = free_ev.back();
            free_ev.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    };
    std::vector<double> step_ms, req_ms, queue_ms;
    int64_t point_steps = 0, steps_total = 0, admission_waits = 0;
    int launches = 0, max_active_seen = 0;
    double active_sum = 0.0;
    double busy_ms = 0.0, host_s = 0.0;   // launches' device time; host time spent enqueuing them
    rvh_status err = RVH_OK;
    const auto t0 = clk::now();
    auto now_s = [&]() { return std::chrono::duration<double>(clk::now() - t0).count(); };
    int done = 0;
    for (int i = 0; i < n; ++i)
        if (results[i].status != RVH_OK) ++done;
    // a character's grid scratch back to the pool (its friction applied, nothing pending)
    auto release = [&](int c) {
        Character& ch = s->chars[c];
        if (ch.bytes) s->pool.give(ch.off, ch.bytes);
        ch.asset->grid[0] = ch.asset->grid[1] = ch.asset->grid[2] = DevBuf{};
        ch.asset->pending = false;
        ch.held = ch.finishing = false;
        ch.off = ch.bytes = 0;
    };
    bool want_space = false;   // an admission waits for pool space held by idle characters
    auto complete = [&](Launch& L) {
        cudaEventSynchronize(L.stop);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, L.start, L.stop);
        busy_ms += ms;
        const double t = now_s();
        for (size_t q = 0; q < L.reqs.size(); ++q) {   // each step's latency: its launch's time
            const int r = L.reqs[q];
            for (int k = 0; k < L.nsteps[q]; ++k) step_ms.push_back(ms);
            results[r].steps_done += L.nsteps[q];
            results[r].max_step_ms = std::max(results[r].max_step_ms, ms);
        }
        for (int r : L.last) {
            results[r].done_s = t;
            req_ms.push_back(1e3 * (t - reqs[r].arrival_s));
            for (size_t k = 0; k < active.size(); ++k)
                if (active[k].req == r) {   // the character keeps its grids and its pending friction
                    s->chars[reqs[r].character].busy = false;
                    active.erase(active.begin() + k);
                    break;
                }
            ++done;
        }
        for (int c : L.finish) release(c);
        for (int r : L.reqs)
            for (Active& ac : active)
                if (ac.req == r) ac.in_flight--;
        point_steps += L.points;
        free_ev.push_back(L.start);
        free_ev.push_back(L.stop);
    };
    while (done < n && err == RVH_OK) {
        const double t = now_s();
        while (next < size_t(n) && reqs[order[next]].arrival_s <= t) {
            if (results[order[next]].status == RVH_OK) waiting.push_back(order[next]);
            ++next;
        }
        // admission: arrival order, skipping requests whose character is busy.  A request takes
        // a slot until its last step is enqueued: launches run in stream order, so no launch
        // steps more than max_active requests, and the next launch can be full while the
        // current one (carrying the last steps of some requests) still runs.
        int stepping = 0;
        for (const Active& ac : active) stepping += ac.remaining > 0 ? 1 : 0;
        for (auto it = waiting.begin(); it != waiting.end() && stepping < s->desc.max_active;) {
            const int r = *it;
            Character& ch = s->chars[reqs[r].character];
            if (ch.busy || ch.finishing) {
                ++it;
                continue;
            }
            Active ac{r, reqs[r].n_steps};
            Asset* a = ch.asset;
            if (a->params.grid_enabled && !ch.held) {
                const size_t gb = a->grid_bytes();
                const size_t one = (gb + 255) & ~size_t(255);
                size_t off = 0;
                if (!s->pool.take(3 * one, &off)) {  // wait for memory; later requests may still fit
                    ++admission_waits;
                    want_space = true;
                    ++it;
                    continue;
                }
                ch.held = true;
                ch.off = off;
                ch.bytes = 3 * one;
                char* base = static_cast<char*>(s->slab.ptr) + off;
                for (int g = 0; g < 3; ++g) {
                    a->grid[g] = DevBuf{base + g * one, gb, s->ctx, false};
                    a->grid_dirty[g] = false;
                }
                cudaMemsetAsync(base, 0, 3 * one, stream);
                a->pending = false;
                a->last_grid = -1;
            }
            ch.busy = true;
            results[r].admit_s = t;
            queue_ms.push_back(1e3 * (t - reqs[r].arrival_s));
            active.push_back(ac);
            ++stepping;
            it = waiting.erase(it);
        }
        max_active_seen = std::max(max_active_seen, stepping);
        // launch one step of every admitted request that still has steps to enqueue
        // Every step is fused: the last step of a request leaves its friction pending in the
        // character's grids, and the character's next request continues from there.  When an
        // admission waits for pool space, idle characters with grids (least recently stepped
        // first) get their pending friction applied in this launch and release their grids.
        std::vector<Asset*> la;
        std::vector<rvh_frame> lf;   // per asset, its steps' frames
        std::vector<int> lm;   // 0: fused steps, 2: apply the pending friction only
        std::vector<int> lsteps;
        Launch L;
        for (Active& ac : active) {
            if (ac.remaining == 0) continue;
            Character& ch = s->chars[reqs[ac.req].character];
            const int n_st = std::min(ac.remaining, s->desc.steps_per_launch);
            for (int k = 0; k < n_st; ++k) {
                rvh_frame f{};
                f.dt = ch.dt;
                f.t = float(double(ch.steps + k + 1) * double(ch.dt));
                if (ch.has_wind) rvh_wind_at(&ch.wind, ch.steps + k, f.t, f.wind);
                lf.push_back(f);
            }
            la.push_back(ch.asset);
            lm.push_back(0);
            lsteps.push_back(n_st);
            L.reqs.push_back(ac.req);
            L.nsteps.push_back(n_st);
            L.points += int64_t(n_st) * ch.asset->n_strands * ch.asset->n_points;
            if (ac.remaining == n_st) L.last.push_back(ac.req);
        }
        const size_t n_requests_in_launch = la.size();   // before any finishing characters join
        if (want_space && int(flight.size()) < s->desc.pipeline_depth) {
            std::vector<int> idle;
            for (int c = 0; c < int(s->chars.size()); ++c) {
                const Character& ch = s->chars[c];
                if (ch.held && !ch.busy && !ch.finishing) idle.push_back(c);
            }
            std::sort(idle.begin(), idle.end(),
                      [&](int x, int y) { return s->chars[x].last_launch < s->chars[y].last_launch; });
            // the grid triples of the waiting requests whose characters hold none, less the
            // space that finishing launches already in flight give back
            size_t need = 0, freed = 0;
            for (int r : waiting) {
                const Character& ch = s->chars[reqs[r].character];
                if (!ch.held && ch.asset->params.grid_enabled)
                    need += 3 * ((ch.asset->grid_bytes() + 255) & ~size_t(255));
            }
            for (const Character& ch : s->chars)
                if (ch.finishing) freed += ch.bytes;
            for (int c : idle) {
                if (freed >= need) break;
                Character& ch = s->chars[c];
                freed += ch.bytes;
                if (!ch.asset->pending) {   // nothing left to apply: the space is free now
                    release(c);
                    continue;
                }
                ch.finishing = true;
                la.push_back(ch.asset);
                lf.push_back(rvh_frame{ch.dt, float(double(ch.steps) * double(ch.dt)), {0.f, 0.f, 0.f}, 0});
                lm.push_back(2);
                lsteps.push_back(1);
                L.finish.push_back(c);
            }
            want_space = false;
        }
        if (!la.empty() && int(flight.size()) < s->desc.pipeline_depth) {
            L.start = get_ev();
            L.stop = get_ev();
            const double h0 = now_s();
            err = dyn_batch_launch_steps(s->batch, la, lsteps, lm, lf, stream, L.start, L.stop);
            host_s += now_s() - h0;
            if (err != RVH_OK) break;
            for (int r : L.reqs) s->chars[reqs[r].character].last_launch = launches + 1;
            for (size_t q = 0; q < L.reqs.size(); ++q)
                for (Active& ac : active)
                    if (ac.req == L.reqs[q]) {
                        ac.remaining -= L.nsteps[q];
                        ac.in_flight++;
                        s->chars[reqs[ac.req].character].steps += L.nsteps[q];
                    }
            for (int n_st : L.nsteps) steps_total += n_st;
            active_sum += double(n_requests_in_launch);
            ++launches;
            flight.push_back(L);
            continue;
        }
        if (!flight.empty()) {
            // a launch is in flight: retire it when it completes (or right away if the pipeline is full)
            if (int(flight.size()) >= s->desc.pipeline_depth || la.empty() ||
                cudaEventQuery(flight.front().stop) == cudaSuccess) {
                complete(flight.front());
                flight.pop_front();
            }
            continue;
        }
        if (next < size_t(n)) {  // idle until the next arrival
            const double wait = reqs[order[next]].arrival_s - now_s();
            if (wait > 2e-4) std::this_thread::sleep_for(std::chrono::duration<double>(wait * 0.5));
            continue;
        }
        if (!waiting.empty() && active.empty()) {  // nothing can ever be admitted
            err = fail(RVH_ERR_BUDGET, "server_run: a request's grid scratch exceeds the server budget");
            for (int r : waiting) results[r].status = RVH_ERR_BUDGET;
            break;
        }
    }
    while (!flight.empty()) {
        complete(flight.front());
        flight.pop_front();
    }
    // the pending friction of every character that still holds grids, in one launch, so the
    // run leaves every asset finished and the pool empty
    if (err == RVH_OK) {
        std::vector<Asset*> la;
        std::vector<rvh_frame> lf;
        std::vector<int> lm;
        Launch L;
        for (int c = 0; c < int(s->chars.size()); ++c) {
            Character& ch = s->chars[c];
            if (!ch.held) continue;
            if (!ch.asset->pending) {
                release(c);
                continue;
            }
            la.push_back(ch.asset);
            lf.push_back(rvh_frame{ch.dt, float(double(ch.steps) * double(ch.dt)), {0.f, 0.f, 0.f}, 0});
            lm.push_back(2);
            L.finish.push_back(c);
        }
        if (!la.empty()) {
            err = dyn_batch_launch(s->batch, la, lf, lm, stream, nullptr, nullptr, nullptr);
            if (err == RVH_OK && cudaStreamSynchronize(stream) != cudaSuccess) err = fail(RVH_ERR_CUDA, "server_run: finish");
        }
        if (err == RVH_OK)
            for (int c : L.finish) release(c);
    }
    for (Active& ac : active)   // only after an error
        s->chars[reqs[ac.req].character].busy = false;
    for (int c = 0; c < int(s->chars.size()); ++c)   // only after an error: drop what is left
        if (s->chars[c].held) release(c);
    for (cudaEvent_t e : free_ev) cudaEventDestroy(e);
    const double wall = now_s();
    rvh_status chk = dyn_batch_check(s->batch);
    if (err == RVH_OK) err = chk;
    if (stats) {
        *stats = rvh_server_stats{};
        stats->requests = n;
        stats->steps = steps_total;
        stats->point_steps = point_steps;
        stats->launches = launches;
        stats->wall_s = wall;
        stats->point_steps_per_s = wall > 0 ? double(point_steps) / wall : 0.0;
        stats->step_ms_p50 = pct(step_ms, 0.50);
        stats->step_ms_p99 = pct(step_ms, 0.99);
        stats->step_ms_p999 = pct(step_ms, 0.999);
        stats->request_ms_p50 = pct(req_ms, 0.50);
        stats->request_ms_p99 = pct(req_ms, 0.99);
        stats->queue_ms_p50 = pct(queue_ms, 0.50);
        stats->queue_ms_p99 = pct(queue_ms, 0.99);
        stats->mean_batch = launches ? active_sum / launches : 0.0;
        stats->max_active = max_active_seen;
        stats->admission_waits = admission_waits;
        stats->scratch_used_bytes = s->pool.used();
        stats->gpu_busy_frac = wall > 0 ? 1e-3 * busy_ms / wall : 0.0;
        stats->host_ms_per_launch = launches ? 1e3 * host_s / launches : 0.0;
    }
    return err;
}

}  // extern "C"
