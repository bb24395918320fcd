"""Benchmark of the GB300 hair step: point-steps/s of the batched step (many
assets, one persistent launch in a CUDA graph) vs the plain step (one launch
sequence per asset), with p50/p99 step latency.

Workload ("batched"): 256 seeded synthetic heads, strands log-uniform in
[512, 65536], points per strand in {8,16,24,32}, lengths U(0.2,1.0), grids
32^3..64^3 (int64 sums), 0-4 ellipsoids + the head sphere, friction 0.05,
repulsion 0.02, wind with gusts.  Inputs (~3.6 GB of Strand records) exceed
L2 (129 MB), so no flush is needed between steps.

  value : device time of the batched launches (CUDA events on the launching
          stream), inputs resident in HBM.
  e2e   : the same step through the C ABI with host data every step: frame
          parameters from pinned host memory (H2D) and every curve point's
          position (xyz) back to host memory (D2H), all inside the timed region
          (rvh_batch_step_read_positions: the step kernel stages the positions).
  full_head : the 100k-strand x 32-point head alone (plain step, and a
          one-asset batch at 8, 16 and 32 lanes per strand), CUDA events.
  error : the FP64 error of the benchmarked step: the CPU legs' sample of
          the workload stepped 120 times through the batched launch (fast
          math), against the FP64 oracle, beside the FP32 twin's (the
          reference shader's arithmetic) and over the well-conditioned strands.
  --impl reference : the oracle's OpenMP C++ restatement of the reference
          shader on the host cores (the reference itself is a Vulkan shader
          and has no CPU implementation), on a bounded sample of the workload.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun (N>1) every rank steps its own 256-head shard of an N x 256-head
workload (weak scaling, no collective on the data path); timing is max over
ranks after a barrier and value sums the ranks' points.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "realtime-vulkan-hair_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "point-steps/s batched+served vs plain on 1 GB300 @1e-3 err; p50/p99 step ms"
BYTES_PER_POINT = 80        # read x,v (32 B) + write x,v,corr (48 B) per point-step
BYTES_PER_CELL = 16         # one clear/flush pass per grid cell-step
# DRAM bytes per algorithmic byte of k_batch, from one ncu capture of the fused
# step on the first 32 heads of the workload (dram__bytes_read.sum +
# dram__bytes_write.sum over 80 B/point + 16 B/cell); traffic grows with points
# and cells, so the full launch's traffic is this ratio times its bytes.  Reads
# are 652.2 MB (the L2 prefetch of each CTA's next item adds about 220 MB of
# reads for a 2 % shorter step), writes 586.1 MB.
TRAFFIC_PER_ALG_BYTE = (652.2 + 586.1) / 833.0


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = os.environ.get("RVH_DIST_BACKEND", "nccl")
        if backend == "nccl" and torch.cuda.is_available():
            # one GPU per rank: NCCL's barrier and the max-over-ranks tensor live on this rank's GPU
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def shard(specs, rank, world):
    """Asset i goes to rank i % world: weak scaling, no data-path collective."""
    return [s for i, s in enumerate(specs) if i % world == rank]


def make_assets(ctx, specs):
    from rvh import api
    assets = []
    for s in specs:
        a = api.Asset(ctx, s.records, s.n_points, rest=s.rest, strand_wind=s.strand_wind)
        a.set_params(s.params)
        a.set_colliders(s.colliders_at(0))
        assets.append(a)
    return assets


def algorithmic_bytes(specs):
    pts = sum(s.n_total_points for s in specs)
    cells = sum(int(np.prod(list(s.params.grid_dims))) for s in specs if s.params.grid_enabled)
    return pts * BYTES_PER_POINT + cells * BYTES_PER_CELL, pts, cells


CPU_SAMPLE_POINTS = 1_500_000   # points of the CPU legs' sample (about 10-30 s of CPU work in all)


def cpu_sample(specs, budget_points=CPU_SAMPLE_POINTS):
    """A bounded sample of the workload for the CPU leg: whole assets taken in
    order until ~budget_points points."""
    out, pts = [], 0
    for s in specs:
        out.append(s)
        pts += s.n_total_points
        if pts >= budget_points:
            break
    return out, pts


def time_cpu(specs, steps, threads):
    from oracle import oracle_ctypes as O
    states = [s.records.copy() for s in specs]
    pts = sum(s.n_total_points for s in specs)
    t0 = time.perf_counter()
    for k in range(steps):
        for st, s in zip(states, specs):
            O.run(st, s.n_points, s.rest, s.params, [s.frame(k)], s.colliders, 1, threads=threads)
    dt = time.perf_counter() - t0
    return pts * steps / dt, dt


def run_served(ctx, args, rank, lanes):
    """1,000 resident characters sized as the batched workload; Poisson arrivals
    at 20k req/s, 1-8 steps each; continuous batching at 1, 4 and 16 requests
    per launch.  Returns ({concurrency: stats}, points, the batched rate of 16
    of these characters in one graph-launched batch, i.e. a launch of the size
    the server builds at concurrency 16).  Per concurrency: the offered load,
    whether it was sustained (served >= 97 % of offered and no queue growth),
    and the queue growth: the slope of each request's queueing delay against
    its arrival time (ms of extra delay per s; about 0 when sustained)."""
    import torch
    from rvh import api, configs
    n_chars = args.characters
    specs = configs.batched(n_assets=n_chars, seed=3)
    assets, out = [], {}
    for s in specs:
        a = api.Asset(ctx, s.records, s.n_points, rest=s.rest)
        a.set_params(s.params)
        a.set_colliders(s.colliders)
        assets.append(a)
    pts = sum(s.n_total_points for s in specs)
    offered = 20000.0 * 4.5 * pts / n_chars
    rng = np.random.default_rng(77)
    for conc in (1, 4, 16):
        srv = api.Server(ctx, max_active=conc, lanes=lanes, pipeline_depth=4, scratch_budget_bytes=24 << 30,
                         steps_per_launch=args.steps_per_launch)
        ids = [srv.add_character(a, wind=s.wind) for a, s in zip(assets, specs)]
        t = np.cumsum(rng.exponential(1.0 / 20000.0, size=args.requests))
        reqs = [(ids[int(rng.integers(0, n_chars))], int(rng.integers(1, 9)), float(ti)) for ti in t]
        st, res, stats = srv.run(reqs)
        d = stats.as_dict()
        d["status"] = st
        d["offered_point_steps_per_s"] = offered
        delay_ms = np.array([1e3 * (r.admit_s - q[2]) for r, q in zip(res, reqs)])
        growth = float(np.polyfit(t, delay_ms, 1)[0]) if len(t) > 1 else 0.0
        d["queue_growth_ms_per_s"] = growth
        d["sustained"] = bool(d["point_steps_per_s"] >= 0.97 * offered and growth < 50.0)
        d["steps_per_launch"] = args.steps_per_launch
        d["pipeline_depth"] = 4
        out[str(conc)] = d
        srv.close()
    # a batch of 16 of the characters, graph-launched: the batched rate at the server's launch size
    sub = assets[:16]
    b = api.Batch(ctx, sub, lanes=lanes)
    frames = [specs[i].frame(0) for i in range(16)]
    st_ = torch.cuda.Stream()
    for k in range(5):
        b.step(frames, stream=st_.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st_)
    for k in range(20):
        b.step(frames, stream=st_.cuda_stream)
    e1.record(st_)
    e1.synchronize()
    b.finish(stream=st_.cuda_stream)
    st_.synchronize()
    sub_pts = sum(specs[i].n_total_points for i in range(16))
    batched16 = sub_pts / (e0.elapsed_time(e1) / 20 * 1e-3)
    b.close()
    for a in assets:
        a.close()
    return out, pts, batched16


def run_full_head(ctx, api, configs, warmup=5, reps=20):
    """The full single head (100,000 strands x 32 points, 64^3 grid, 4
    ellipsoids + the head sphere, wind with gusts): per-step device time by
    CUDA events on the launching stream, through the plain step (rvh_step:
    one launch sequence) and through a one-asset batch (persistent launch in a
    CUDA graph).  The records (154 MB) are a little larger than L2 (129 MB)."""
    import torch
    spec = configs.full_head()
    st = torch.cuda.Stream()
    n_pts = spec.n_strands * spec.n_points
    cells = int(np.prod(list(spec.params.grid_dims)))
    alg = 80 * n_pts + 16 * cells
    peak, _ = load_peaks()
    out = {"workload": "100k strands x 32 points, 64^3 grid, 4 ellipsoids + head sphere, wind with gusts",
           "points_per_step": n_pts, "grid_cells": cells}

    def timed(step_fn):
        for k in range(warmup):
            step_fn(k)
        st.synchronize()
        per = []
        for k in range(warmup, warmup + reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            step_fn(k)
            e1.record(st)
            e1.synchronize()
            per.append(e0.elapsed_time(e1))
        per.sort()
        ms = sum(per) / len(per)
        gbs = alg / (ms * 1e-3) / 1e9
        return {"ms_per_step": ms, "p50_step_ms": per[len(per) // 2], "p99_step_ms": per[-1],
                "point_steps_per_s": n_pts / (ms * 1e-3),
                "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                             "bytes_per_step": alg}}

    def make(lanes=0):
        a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest, strand_wind=spec.strand_wind, lanes=lanes)
        a.set_params(spec.params)
        a.set_colliders(spec.colliders_at(0))
        return a

    plain_by_lanes = {}
    for lanes in (0, 4, 8, 16, 32):   # 0: the asset's default for its point count
        a = make(lanes)

        def plain(k):
            a.set_colliders(spec.colliders_at(k))
            a.step(spec.frame(k), stream=st.cuda_stream)
        plain_by_lanes[lanes] = timed(plain)
        a.close()
    out["plain"] = plain_by_lanes[0]
    out["plain_ms_by_lanes"] = {str(k): v["ms_per_step"] for k, v in plain_by_lanes.items() if k}
    by_lanes = {}
    for lanes in (8, 16, 32):   # every strand has 32 points: the lane count is tried, not assumed
        a = make()
        b = api.Batch(ctx, [a], lanes=lanes)

        def batched(k):
            a.set_colliders(spec.colliders_at(k))
            b.step([spec.frame(k)], stream=st.cuda_stream)
        by_lanes[lanes] = timed(batched)
        b.close()
        a.close()
    best = min(by_lanes, key=lambda x: by_lanes[x]["ms_per_step"])
    out["batched"] = dict(by_lanes[best], lanes_per_strand=best)
    out["batched_ms_by_lanes"] = {str(k): v["ms_per_step"] for k, v in by_lanes.items()}
    return out


def run_tess(ctx, api, configs, warmup=3, reps=10):
    """Strand tessellation of the 100k-strand head (32 points) after a few
    steps, with the reference's levels (12 isolines x 42 segments): device
    time by CUDA events on the launching stream.  `ms`: pinned roots (the
    reference's case), so the per-strand sd profiles come from the cache;
    `ms_roots_moving`: a head motion before every call, every profile recomputed."""
    import torch
    spec = configs.full_head()
    a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    for k in range(3):
        a.step(spec.frame(k))
    ctx.synchronize()
    d = api.tess_desc_reference()
    ns, per = spec.n_strands, d.n_lines * (d.n_segments + 1)
    out = torch.empty((ns * per * 4,), dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()
    for _ in range(warmup):
        a.tessellate(out.data_ptr(), None, desc=d, stream=st.cuda_stream)
    st.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        a.tessellate(out.data_ptr(), None, desc=d, stream=st.cuda_stream)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # the same with the roots moving before every call (a head motion and a step
    # in between): no cached sd profile applies, each call recomputes them all
    pose = np.eye(4, dtype=np.float32)
    moving = []
    for k in range(warmup + reps):
        pose[1, 3] = np.float32(0.001 * (k + 1))
        a.set_head_transform(pose)
        a.step(spec.frame(3 + k), stream=st.cuda_stream)
        e0.record(st)
        a.tessellate(out.data_ptr(), None, desc=d, stream=st.cuda_stream)
        e1.record(st)
        e1.synchronize()
        if k >= warmup:
            moving.append(e0.elapsed_time(e1))
    ms_moving = sum(moving) / len(moving)
    a.close()
    vertices = ns * per
    alg = vertices * 16 + ns * spec.n_points * 16      # vertex writes + position reads
    peak, _ = load_peaks()
    gbs = alg / (ms * 1e-3) / 1e9
    return {"workload": "100k strands x 32 points (the full head), 12 isolines x 42 segments per strand",
            "vertices": vertices, "ms": ms, "vertices_per_s": vertices / (ms * 1e-3),
            "ms_roots_moving": ms_moving,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "bytes_per_launch": alg}}


def run_shade(ctx, api, configs, warmup=3, reps=10):
    """The shadow, opacity and hair passes over the tessellated 100k-strand head
    (12 isolines x 42 segments, 51.6 M vertices) with the reference's cameras
    and 1080 x 720 maps: device time of rvh_asset_shade by CUDA events on the
    launching stream; then the rasterised camera image (rvh_asset_render_hair).  Algorithmic bytes: each vertex read by the three passes
    (3 x 16 B), its colour written (16 B), the segment frames read once, and
    the maps cleared, finished and read back once (depth 4 B, layers 16 B per
    texel, three times)."""
    import torch
    spec = configs.full_head()
    a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    for k in range(3):
        a.step(spec.frame(k))
    ctx.synchronize()
    td, sd = api.tess_desc_reference(), api.shade_desc_reference()
    ns, per = spec.n_strands, td.n_lines * (td.n_segments + 1)
    vertices = ns * per
    texels = sd.map_width * sd.map_height
    vert = torch.empty((vertices * 4,), dtype=torch.float32, device="cuda")
    frames = torch.empty((ns * (spec.n_points - 1) * 12,), dtype=torch.float32, device="cuda")
    depth = torch.empty((texels,), dtype=torch.float32, device="cuda")
    opac = torch.empty((texels * 4,), dtype=torch.float32, device="cuda")
    col = torch.empty((vertices * 4,), dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()
    a.tessellate(vert.data_ptr(), frames.data_ptr(), desc=td, stream=st.cuda_stream)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(desc):
        def once():
            a.shade(vert.data_ptr(), frames.data_ptr(), depth.data_ptr(), opac.data_ptr(), col.data_ptr(),
                    tess_desc=td, shade_desc=desc, stream=st.cuda_stream)

        for _ in range(warmup):
            once()
        st.synchronize()
        e0.record(st)
        for _ in range(reps):
            once()
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    # the light maps as one texel per vertex (the cheap mode), then as the
    # reference draws them (hair.geom's quads); the image uses the latter
    ms_vertex_maps = timed(api.shade_desc_reference(map_mode=api.SHADE_MAPS_VERTICES))
    ms = timed(sd)
    covered = int((depth < 1).sum().item())
    # the camera image: hair.geom's quads rasterised at the window size, 1080 x 720
    W, H = 1080, 720
    image = torch.empty((W * H * 4,), dtype=torch.float32, device="cuda")

    ids = torch.empty((W * H,), dtype=torch.int32, device="cuda")

    def render(desc=sd):
        a.render_hair(vert.data_ptr(), frames.data_ptr(), depth.data_ptr(), opac.data_ptr(), W, H, image.data_ptr(),
                      ids.data_ptr(), tess_desc=td, shade_desc=desc, stream=st.cuda_stream)

    def timed_render(desc):
        for _ in range(warmup):
            render(desc)
        st.synchronize()
        e0.record(st)
        for _ in range(reps):
            render(desc)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    # the image as the reference pipeline blends it (sd.image_mode = blend), and with the nearest fragment only
    render_nearest_ms = timed_render(api.shade_desc_reference(image_mode=api.IMAGE_NEAREST))
    render_ms = timed_render(sd)
    pixels = int((ids != -1).sum().item())
    # the reference's frame: shadow + opacity passes (maps from the quads) and the hair pass (the image)

    def frame():
        a.shade(vert.data_ptr(), frames.data_ptr(), depth.data_ptr(), opac.data_ptr(), 0, tess_desc=td,
                shade_desc=sd, stream=st.cuda_stream)
        render()

    for _ in range(warmup):
        frame()
    st.synchronize()
    e0.record(st)
    for _ in range(reps):
        frame()
    e1.record(st)
    e1.synchronize()
    frame_ms = e0.elapsed_time(e1) / reps
    a.close()
    alg = vertices * 64 + ns * (spec.n_points - 1) * 48 + texels * 20 * 3
    peak, _ = load_peaks()
    gbs = alg / (ms * 1e-3) / 1e9
    return {"workload": "100k strands x 32 points (the full head), 12 isolines x 42 segments, 1080 x 720 maps "
                        "rasterised from hair.geom's quads in the light's view",
            "vertices": vertices, "covered_texels": covered, "ms": ms, "vertices_per_s": vertices / (ms * 1e-3),
            "ms_vertex_maps": ms_vertex_maps,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "bytes_per_launch": alg},
            "render": {"workload": "hair.geom quads of every isoline segment rasterised into 1080 x 720, "
                                   "shaded by hair.frag",
                       "segments": ns * td.n_lines * td.n_segments, "ms": render_ms, "covered_pixels": pixels,
                       "image_mode": "blend in primitive order (the reference pipeline)",
                       "ms_nearest_fragment": render_nearest_ms},
            "frame_ms": frame_ms}


def run_error(ctx, api, specs, lanes, steps=120):
    """FP64 error of the benchmarked step: the CPU legs' sample of the batched
    workload (its leading assets), fresh from the generator, stepped `steps`
    times through the batched launch (fast math, the timed lane count), then
    compared with the FP64 oracle over the same frames.  The FP32 twin (the
    reference shader's own arithmetic) is reported beside it, and both again
    over the well-conditioned strands (oracle/errors.py)."""
    from oracle import errors as E
    from oracle import oracle_ctypes as O
    sample, pts = cpu_sample(specs)
    assets = make_assets(ctx, sample)
    b = api.Batch(ctx, assets, lanes=lanes)
    for k in range(steps):
        b.step([s.frame(k) for s in sample])
    b.finish()
    b.check()
    got = [a.read() for a in assets]
    b.close()
    for a in assets:
        a.close()
    thr = O.max_threads()
    ef, et, wf, wt = [], [], [], []
    seg, n_well, n_all = 0.0, 0, 0
    for g, s in zip(got, sample):
        L = E.lengths(s.rest, s.n_points)
        ref = E.run_spec(s, steps, np.float64, thr)
        twin = E.run_spec(s, steps, np.float32, thr)
        well = E.spread(s, steps, ref, thr) <= 1e-4
        e_f, e_t = E.point_errors(g, ref, s.n_points, L), E.point_errors(twin, ref, s.n_points, L)
        ef.append(e_f.reshape(-1))
        et.append(e_t.reshape(-1))
        wf.append(e_f[well].reshape(-1))
        wt.append(e_t[well].reshape(-1))
        seg = max(seg, E.segment_error(g, s.rest, s.n_points))
        n_well += int(well.sum())
        n_all += s.n_strands
    cat = np.concatenate
    return {"steps": steps, "vs": "FP64 oracle", "unit": "|x - x_fp64| / strand length, per curve point",
            "sample": "first %d assets (%d points) of the workload, batched launch, fast math, lanes %d"
                      % (len(sample), pts, lanes),
            "fast": E.summary(cat(ef)), "reference_fp32": E.summary(cat(et)),
            "well_conditioned": {"strands": n_well, "of": n_all, "fast": E.summary(cat(wf)),
                                 "reference_fp32": E.summary(cat(wt))},
            "seg_len_max": seg,
            "note": "reference_fp32 = the oracle's FP32 twin, bit-identical to the reference shader's arithmetic; "
                    "well-conditioned = FP64 spread of a 1e-7 L initial perturbation <= 1e-4 L after the same steps"}


def run_adjoint(ctx, api, configs, reps=3):
    """The differentiable step: 4,096 strands x 32 points over 60 steps, the FP32
    adjoint of the tip loss with checkpoints every 10 steps (forward, per-segment
    recompute, reverse), wall time per call (synchronous) and per step."""
    spec, targets = configs.adjoint_case(n_strands=4096, n_points=32)
    a = api.Asset(ctx, spec.records, spec.n_points, rest=spec.rest, strand_wind=spec.strand_wind)
    a.set_params(spec.params)
    a.set_colliders(spec.colliders)
    frames = [spec.frame(k) for k in range(60)]
    a.adjoint(frames, targets)   # warm-up
    t0 = time.perf_counter()
    for _ in range(reps):
        a.write(spec.records)
        a.adjoint(frames, targets)
    ms = (time.perf_counter() - t0) * 1e3 / reps
    a.close()
    pts = spec.n_strands * spec.n_points
    return {"workload": "%d strands x 32 points, 60 steps, checkpoints every 10, tip loss" % spec.n_strands,
            "ms": ms, "ms_per_step": ms / 60, "point_steps_per_s": pts * 60 / (ms * 1e-3)}


def cpu_sample_count(n_assets, budget_points=CPU_SAMPLE_POINTS):
    """How many leading assets of the batched workload cpu_sample takes."""
    from rvh import configs
    pts = 0
    for i, (ns, n, _, _) in enumerate(configs.batched_sizes(n_assets)):
        pts += ns * n
        if pts >= budget_points:
            return i + 1
    return n_assets


def run_reference(args, rank, world):
    """--impl reference: the oracle's OpenMP restatement on the host cores.
    The workload sample comes from the oracle's own statement of the seeded
    generator (oracle/scene_oracle.hpp), so this process never maps the CUDA
    library; it is byte for byte the sample the GPU arm's cpu_baseline times."""
    if rank != 0:
        return
    from oracle import build as oracle_build
    oracle_build.build()
    from oracle import oracle_ctypes as O
    from rvh import configs
    specs = configs.batched(n_assets=args.assets, gen=O.SceneGen(), indices=range(cpu_sample_count(args.assets)))
    sample, pts = cpu_sample(specs)
    threads = O.max_threads()
    time_cpu(sample, 1, threads)  # warm-up
    per_step = []
    for k in range(args.steps):
        v, dt = time_cpu(sample, 1, threads)
        per_step.append(dt)
    value = pts * len(per_step) / sum(per_step)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "point-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(per_step),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": "batched: 256 heads, strands log-uniform 512..65536, 8..32 points, "
                                   "32^3..64^3 grids", "sample_points": pts},
            "cpu_baseline": {"value": value, "unit": "point-steps/s", "cores": threads, "kind": "port",
                             "sample": "first %d assets (%d points) of the batched workload, %d steps, FP32 "
                                       "OpenMP over strands" % (len(sample), pts, args.steps)},
            "e2e": {"value": value, "unit": "point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--assets", type=int, default=256)
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-tess", action="store_true")
    ap.add_argument("--no-full-head", action="store_true")
    ap.add_argument("--no-shade", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-error", action="store_true")
    ap.add_argument("--characters", type=int, default=1000)
    ap.add_argument("--requests", type=int, default=3000)
    ap.add_argument("--steps-per-launch", type=int, default=3)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import __graft_entry__
    __graft_entry__.build()
    from rvh import api, configs

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    # weak scaling: every rank steps a full workload of args.assets heads (rank r takes
    # heads r, r + N, ... of N * args.assets), with no collective on the data path
    all_specs = configs.batched(n_assets=args.assets * world)
    specs = shard(all_specs, rank, world)
    ctx = api.Context(device=dev, math=api.MATH_FAST)
    assets = make_assets(ctx, specs)
    frames = [[s.frame(k) for s in specs] for k in range(args.warmup + args.steps)]
    tuned = None
    if args.lanes == 0 and not args.no_tune:
        t0 = time.perf_counter()
        tr = api.tune(ctx, assets, frames[0], steps=2)
        tuned = {"lanes_per_strand": tr.lanes_per_strand, "strands_per_tile": tr.strands_per_tile,
                 "best_ms": tr.best_ms, "seconds": time.perf_counter() - t0,
                 "tried": [{"lanes": l, "tile": t, "ms": round(m, 3)} for l, t, _, m in tr.table()]}
    batch = api.Batch(ctx, assets, lanes=args.lanes)
    info = batch.info()
    alg_bytes, pts, cells = algorithmic_bytes(specs)

    # ---- batched step, device time ----
    for k in range(args.warmup):
        batch.step(frames[k])
    ctx.synchronize()
    batch.check()
    barrier(world)
    clocks = ClockSampler(dev)
    clocks.start()
    batch.timing(True)
    batch.read_timing()
    t0 = time.perf_counter()
    for k in range(args.steps):
        batch.step(frames[args.warmup + k])
    ctx.synchronize()
    host_s = time.perf_counter() - t0
    dev_ms, launches = batch.read_timing()
    batch.timing(False)
    clk = clocks.stop()
    batch.check()
    step_ms = dev_ms / max(1, launches)
    step_ms = max_over_ranks(step_ms, world)
    total_pts = int(sum_over_ranks(pts, world))   # every rank's points of one step
    value = total_pts / (step_ms * 1e-3)

    # per-step latency distribution (each launch timed separately)
    lat = []
    batch.timing(True)
    for k in range(min(args.steps, 20)):
        batch.step(frames[k % len(frames)])
        ms, _ = batch.read_timing()
        lat.append(ms)
    batch.timing(False)
    # the last fused step's pending gather + friction, applied once at the end of a run
    ctx.synchronize()
    t0 = time.perf_counter()
    batch.finish()
    ctx.synchronize()
    finish_ms = (time.perf_counter() - t0) * 1e3
    # the benchmarked state after every step of this run: finite, clamped, inextensible
    hs = [a.health() for a in assets]
    health = {"assets": len(hs), "nonfinite": int(sum(h.nonfinite for h in hs)),
              "max_speed": float(max(h.max_speed for h in hs)) if hs else 0.0,
              "max_length_error": float(max(h.max_length_error for h in hs)) if hs else 0.0}

    # ---- plain step: one launch sequence per asset, no graph ----
    plain_value, plain_ms = None, None
    if not args.no_plain:
        for k in range(2):
            for a, s in zip(assets, specs):
                a.step(s.frame(k))
        ctx.synchronize()
        nplain = max(3, min(args.steps, 10))
        t0 = time.perf_counter()
        for k in range(nplain):
            for a, s in zip(assets, specs):
                a.step(s.frame(k))
        ctx.synchronize()
        plain_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / nplain, world)
        plain_value = total_pts / (plain_ms * 1e-3)

    # ---- e2e through the C ABI with host buffers ----
    # every step: frame tables host->device (inside the step call) and every
    # curve point's position (xyz, 12 B) device->host.  rvh_batch_step_read_positions:
    # the step kernel writes each new position into a staging slot as it stores the
    # record, and a second stream copies it so the copy of step k overlaps step k+1.
    # For comparison, the same with a separate packing pass after each step
    # (rvh_batch_step + rvh_batch_read_positions_async).
    pos_bytes = pts * 12
    pinned = [api.PinnedBuffer(pos_bytes) for _ in range(2)]
    h2d = batch.h2d_bytes_per_step()
    ne2e = max(3, min(args.steps, 10))

    def e2e_run(fused):
        def one(k):
            if fused:
                batch.step_read_positions(frames[k], pinned[k % 2].ptr, pos_bytes)
            else:
                batch.step(frames[k])
                batch.read_positions_async(pinned[k % 2].ptr, pos_bytes)
        for k in range(2):
            one(k)
        batch.positions_wait()
        ctx.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for k in range(ne2e):
            one(k)
        batch.positions_wait()
        ctx.synchronize()
        return max_over_ranks((time.perf_counter() - t0) * 1e3 / ne2e, world)

    e2e_pack_ms = e2e_run(False)
    e2e_ms = e2e_run(True)
    e2e_value = total_pts / (e2e_ms * 1e-3)
    d2h = pos_bytes
    for p_ in pinned:
        p_.close()

    # ---- CPU baseline on a bounded sample (rank 0, N=1 only) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import oracle_ctypes as O
        sample, spts = cpu_sample(specs)
        threads = O.max_threads()
        v, dt = time_cpu(sample, 3, threads)
        cpu = {"value": v, "unit": "point-steps/s", "cores": threads, "kind": "port",
               "sample": "first %d assets (%d points) of the workload, 3 steps, FP32 OpenMP restatement "
                         "of the reference shader" % (len(sample), spts)}

    err = None
    if rank == 0 and world == 1 and not args.no_error:
        err = run_error(ctx, api, specs, info["lanes"])

    full = None
    if world == 1 and not args.no_full_head:
        full = run_full_head(ctx, api, configs)
    tess = None
    if world == 1 and not args.no_tess:
        tess = run_tess(ctx, api, configs)
    shade = None
    if world == 1 and not args.no_shade:
        shade = run_shade(ctx, api, configs)
    adjoint = None
    if world == 1 and not args.no_adjoint:
        adjoint = run_adjoint(ctx, api, configs)

    served, served_pts, batched16 = None, None, None
    if not args.no_served and world == 1:
        batch.close()
        for a in assets:
            a.close()
        assets, batch = [], None
        served, served_pts, batched16 = run_served(ctx, args, rank, info["lanes"])
        for d in served.values():
            d["vs_batched"] = d["point_steps_per_s"] / value
            d["vs_batched_16_characters"] = d["point_steps_per_s"] / batched16

    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (step_ms * 1e-3) / 1e9
    if rank == 0:
        lat_sorted = sorted(lat)
        line = {
            "metric": METRIC, "value": value, "unit": "point-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators, no dataset)",
            "config": {"workload": "batched: %d heads per GPU (%d in all), strands log-uniform 512..65536, "
                                   "points {8,16,24,32}, lengths U(0.2,1), grids 32^3..64^3, 0-4 ellipsoids"
                                   % (args.assets, args.assets * world),
                       "points_per_step": total_pts, "grid_cells": cells, "lanes_per_strand": info["lanes"],
                       "work_items": info["items"], "ctas": info["ctas"],
                       "l2": "inputs (%.1f GB) larger than L2; no flush" % (pts * 48 / 1e9),
                       "math": "fast"},
            "p50_step_ms": lat_sorted[len(lat_sorted) // 2], "p99_step_ms": lat_sorted[-1],
            "finish_ms": finish_ms, "health": health, "tuner": tuned,
            "plain": {"value": plain_value, "ms_per_step": plain_ms,
                      "speedup_batched_vs_plain": (value / plain_value) if plain_value else None},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": alg_bytes * TRAFFIC_PER_ALG_BYTE,
                         "traffic_source": "ncu DRAM bytes of k_batch on the first 32 heads, scaled by "
                                           "algorithmic bytes",
                         "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                         "fallback 6.8 TB/s"},
            "e2e": {"value": e2e_value, "unit": "point-steps/s", "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "api": "rvh_batch_step_read_positions",
                    "ms_per_step_with_packing_pass": e2e_pack_ms},
            "error": err,
            "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches), "tessellation": tess,
            "shading": shade, "adjoint": adjoint, "full_head": full,
            "served": None if served is None else {
                "workload": "%d resident characters sized as the batched workload (%d points), Poisson "
                            "arrivals 20k req/s, 1-8 steps per request, %d requests per run" % (
                                args.characters, served_pts, args.requests),
                "batched_16_characters_point_steps_per_s": batched16,
                "by_concurrency": served},
        }
        print(json.dumps(line), flush=True)
    if batch is not None:
        batch.close()
    for a in assets:
        a.close()
    ctx.close()


if __name__ == "__main__":
    main()
