#!/usr/bin/env python3
"""Benchmark of the chunk generation + meshing path (one JSON line on stdout).

Headline workload: 32x32 = 1024 chunks of 16^3 with a 2-D fBm heightmap (4 octaves,
lacunarity 2, gain 0.5, f = 1/128, seed 7, amplitude 48, base 8), meshed in the vertex
layout (4 x 24-byte vertices + 6 u32 indices per face). One step = one pass of the fused
generation + meshing path over the whole batch, replayed from a captured CUDA graph with
the autotuned launch shape and output slab. The same line also carries:
  - plain_per_chunk: the plain per-chunk GPU path (one generate + one mesh launch per
    chunk), replayed from a captured graph so that no host work is timed;
  - e2e: the same batch through vox_gen_mesh_host with page-locked host buffers;
  - mesh_from_occupancy: the rebuild path (vox_mesh_batch over resident occupancy),
    byte-compared with the fused output;
  - stress / density: the 2048 x 64^3 Bernoulli and the 4096 x 32^3 3-D density workloads
    measured the same way, with their own clocks, rooflines and CPU baselines;
  - serving: 10,000 real-time frames of the streaming engine (p50/p99 request-to-mesh
    latency, overall and after the first view fill) and its unpaced capacity.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

--impl reference times the reference's CPU chunk builder restated as the C oracle
(Chunk::new + create_mesh per chunk on all host threads, one chunk per task); the
reference itself is Rust and cannot be built here.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "wgpu-voxel-engine_gb300"), os.path.join(ROOT, "oracle")]

METRIC = "chunks/s gen+mesh (batched vs per-chunk GPU, bit-exact); p50/p99 chunk latency"
WORKLOAD_TEXT = {
    "heightmap": "heightmap-fbm: 32x32 chunks of 16^3 (1024 chunks), 2-D fBm 4 oct f=1/128 seed 7 "
                 "amp 48 base 8, reference culling, vertex layout",
    "plain": "plain-perlin: 8x8 chunks of 32^3 around the origin, 2-D Perlin perm seed 42 f=1/64 "
             "amp 12 base 4, reference culling, vertex layout",
    "density": "density-fbm3: 16x16x16 chunks of 32^3 (4096), 3-D fBm 3 oct f=1/96 seed 1234, "
               "solid iff fbm-(y-256)/64>0, reference culling, vertex layout",
    "stress": "bernoulli-stress: 2048 isolated chunks of 64^3, Bernoulli(0.5) splitmix64(99^index), "
              "vertex layout",
}
SERVING_TEXT = ("serving: simulated camera 20 u/s + 90 deg/s yaw, 60 frames/s, heightmap-fbm 16^3 "
                "chunks, view radius 24, 24 GB LRU cache")
L2_FLUSH_BYTES = 256 << 20

# Per-launch figures of one ncu capture of each kernel on each workload (the command and
# the other metrics are in the named summary under profiles/). traffic = dram bytes read +
# written by one launch; for stress the capture ran on 48 chunks and the figure is scaled
# to the launch's chunk count (DRAM bytes grow with the faces written).
NCU = {
    ("k_mesh_batch_overlap", "heightmap"): {
        "traffic": 7112704, "warp_instructions": 18389229, "chunks": 1024,
        "summary": "profiles/k_mesh_batch_overlap_heightmap.md"},
    ("k_mesh_batch_phased", "heightmap"): {
        "traffic": 6473984, "warp_instructions": 16886488, "chunks": 1024,
        "summary": "profiles/k_mesh_batch_phased_heightmap.md"},
    ("k_mesh_batch_overlap", "density"): {
        "traffic": 658092032, "warp_instructions": 707898692, "chunks": 4096,
        "summary": "profiles/k_mesh_batch_overlap_density.md"},
    # staged halos: the traffic of one step's whole sequence (coordinate map, neighbour
    # lookup, k_generate, k_generate_planes, meshing from the pool)
    ("k_mesh_batch_overlap staged", "density"): {
        "traffic": 650796032, "chunks": 4096, "per_step": True,
        "summary": "profiles/staged_halo_density.md"},
    ("k_mesh_batch_phased staged", "density"): {
        "traffic": 688578304, "chunks": 4096, "per_step": True,
        "summary": "profiles/staged_halo_density.md"},
    ("k_mesh_batch_overlap", "stress"): {
        "traffic": 47944924160, "chunks": 1024, "scaled_from_chunks": 48,
        "summary": "profiles/k_mesh_batch_overlap_stress.md"},
    ("k_mesh_batch_phased", "stress"): {
        "traffic": 47919420245, "chunks": 1024, "scaled_from_chunks": 48,
        "summary": "profiles/k_mesh_batch_phased_stress.md"},
}


def parse_args(argv=None):
    """The bench's command line (the driver's --gpus/--steps/--warmup, and sub-run knobs)."""
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=400)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=list(WORKLOAD_TEXT) + ["serving"], default="heightmap")
    p.add_argument("--layout", choices=["vertex", "instanced"], default="vertex")
    p.add_argument("--cpu-seconds", type=float, default=8.0,
                   help="wall time of the CPU-baseline sample of the headline workload")
    p.add_argument("--e2e-steps", type=int, default=50)
    p.add_argument("--plain-steps", type=int, default=3)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--no-graph", action="store_true",
                   help="launch through vox_gen_mesh_batch instead of replaying a captured graph")
    p.add_argument("--tuning", default=None,
                   help="force a launch shape 'threads,stage_faces,ctas_per_sm[,schedule[,slab[,halo]]]' "
                        "(schedule 0 look-back, 1 phased, 2 overlap; halo 0 regenerated, 1 pool; "
                        "no autotune)")
    p.add_argument("--no-suite", action="store_true",
                   help="headline workload only (no stress / density / serving sub-runs)")
    p.add_argument("--suite-steps", type=int, default=0, help="timed steps of the sub-runs (0: --steps)")
    p.add_argument("--serving-frames", type=int, default=10000,
                   help="real-time frames of the serving sub-run (0: skip)")
    p.add_argument("--capacity-chunks", type=int, default=65536,
                   help="chunks of the unpaced serving capacity run (0: skip)")
    p.add_argument("--frames", type=int, default=10000, help="--workload serving: frames")
    p.add_argument("--paced", action="store_true", help="--workload serving: real-time 60 fps")
    p.add_argument("--tune-iters", type=int, default=5)
    p.add_argument("--limit-chunks", type=int, default=0,
                   help="use only the first K chunks of the workload (small cases for profilers)")
    p.add_argument("--clock-hold", type=float, default=0.3,
                   help="seconds of untimed replays before the timed steps (clock sampling)")
    return p.parse_args(argv)


def dist_info():
    """(rank, world size, local rank) from the torchrun environment (0, 1, 0 alone)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def shard_workload(wl, rank: int, world: int):
    """Weak scaling: every rank gets a batch of the same size and shape, shifted in x by
    64 chunks per rank (Bernoulli: its own chunk-index range). No data exchange."""
    import voxgpu
    if world <= 1:
        return wl
    if wl.isolated:
        return voxgpu.Workload(wl.name, wl.cfg_kwargs, wl.coords, wl.index_base + rank * len(wl.coords),
                               wl.isolated)
    coords = tuple((x + 64 * rank, y, z) for (x, y, z) in wl.coords)
    return voxgpu.Workload(wl.name, wl.cfg_kwargs, coords, wl.index_base, wl.isolated)


def limited(wl, k: int):
    """The first k chunks of a workload (all of them for k <= 0)."""
    import voxgpu
    if k <= 0 or k >= len(wl.coords):
        return wl
    return voxgpu.Workload(wl.name, wl.cfg_kwargs, tuple(wl.coords[:k]), wl.index_base, wl.isolated)


def config_of(name: str, layout: str, limit: int = 0):
    """The workload description both arms print (the same dict, so the lines compare)."""
    import voxgpu
    wl = limited(voxgpu.workload(name), limit)
    return {"workload": WORKLOAD_TEXT[name], "chunks": len(wl.coords),
            "chunk_size": wl.cfg_kwargs["chunk_size"], "layout": layout}


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the GPU works."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        samples = []
        for ln in self.lines:
            parts = [s.strip() for s in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                samples.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in samples for i, v in enumerate(r)
                          if v.lower() == "active"})
        return {"sm_mhz": statistics.median(s[0] for s in samples),
                "sm_max_mhz": max(s[1] for s in samples), "reasons": reasons,
                "samples": len(samples)}


def load_peak():
    """The measured HBM copy rate (GB/s) and its source, else the fallback figure."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# Warp-instruction issue capacity: 152 SMs x 4 schedulers x 2.07 GHz (nominal).
ISSUE_PEAK = 152 * 4 * 2.07e9

# FP32 operations of one noise sample-octave in the noise formula (the oracle's
# or_noise2_f32 / or_noise3_f32 plus one fBm step): floors, fractional parts, fades
# (7 each), corner gradients (2-D: 2 mul + 1 add; 3-D: 3 mul + 2 add), lerps (3 each),
# the coordinate scaling and the fBm update (sum, amp, f).
NOISE_OPS = {2: 2 + 2 + 14 + 2 + 4 * 3 + 3 * 3 + 2 + 4, 3: 3 + 3 + 21 + 3 + 8 * 5 + 7 * 3 + 3 + 4}
# FP32 lane operations the kernels execute per sample-octave. The 2-D heightmap path
# evaluates the whole formula per column. The 3-D lattice-table paths compute the per-axis
# parts (floors, fractions, fades) once per coordinate: per sample they execute the corner
# dot products, the lerps and the fBm sum (8 x 5 + 7 x 3 + 3 = 64). The 32^3 lane = z path
# holds g.y * y and g.z * z per corner record and evaluates corner pairs as f32x2 (two lanes
# per instruction): 4 dot pairs (1 mul + 2 adds), 2 x-lerp pairs and 1 y-lerp pair
# (3 each) = 21 x 2, the z lerp and the sum (5), and the record products (8 pairs, at
# least once per 8 samples: 2) = 49.
NOISE_EXEC_OPS = {"2d": NOISE_OPS[2], "3d_table": 64, "3d_lane_z": 49}
# FP32 lane rate: 152 SMs x 128 lanes x 2.07 GHz, one operation per lane per cycle (an f32x2
# instruction is two). Nominal: the measured peaks file has no FP32 figure.
FP32_OPS_NOMINAL = 152 * 128 * 2.07e9
FP32_PEAK_SOURCE = ("nominal FP32 lane rate (152 SMs x 128 lanes x 2.07 GHz, FMA contraction off); "
                    "the measured-peaks file has no FP32 figure")


def own_noise_ops(cfg):
    """Executed FP32 lane operations per sample-octave of a chunk's own samples."""
    if cfg.gen.kind == 0:
        return NOISE_EXEC_OPS["2d"]
    return NOISE_EXEC_OPS["3d_lane_z" if cfg.chunk_size == 32 else "3d_table"]


def noise_report(wl, cfg, masks, ms_per_step):
    """FP32 throughput of the noise in one step: samples x octaves x the lane operations
    their path executes, against the FP32 lane rate; beside it the rate in formula operations
    (the per-sample formula's count at the same sample rate)."""
    N = cfg.chunk_size
    g = cfg.gen
    n_chunks = len(masks)
    if g.kind == 0:    # heightmap: 2-D noise per column, (N + 2)^2 - 4 columns with halo
        samples, dim = (N + 2) ** 2 - 4, 2
        total = n_chunks * samples
        ops = total * g.octaves * NOISE_EXEC_OPS["2d"]
    elif g.kind == 1:  # density: 3-D noise per voxel and per halo voxel of a loaded neighbour
        samples, dim = N ** 3, 3
        used = 0x3F if cfg.cull_mode == 1 else 0x0F
        halo = sum(bin(m & used).count("1") for m in masks) * N * N
        total = n_chunks * samples + halo
        ops = (n_chunks * samples * own_noise_ops(cfg) + halo * NOISE_EXEC_OPS["3d_table"]) * g.octaves
        samples = total / n_chunks
    else:
        return None
    achieved = ops / (ms_per_step / 1e3)
    formula = total * g.octaves * NOISE_OPS[dim] / (ms_per_step / 1e3)
    return {"samples_per_chunk": samples, "octaves": g.octaves,
            "exec_ops_per_sample_octave": ops / (total * g.octaves),
            "formula_ops_per_sample_octave": NOISE_OPS[dim],
            "achieved_tops": achieved / 1e12, "peak_tops": FP32_OPS_NOMINAL / 1e12,
            "peak_source": FP32_PEAK_SOURCE, "frac": achieved / FP32_OPS_NOMINAL,
            "formula_tops": formula / 1e12,
            "note": "executed lane operations of the step's noise over the whole step time (the "
                    "launch also culls and emits); formula_tops counts the per-sample formula's "
                    "operations at the same sample rate"}


def cpu_baseline(wl, cfg, masks, seconds: float, threads: int = 0):
    """The oracle restatement of the reference CPU chunk builder on `threads` host threads
    (0: all), repeated over the workload (or a prefix of it) for about `seconds`."""
    import vox_oracle
    threads = threads or os.cpu_count() or 1
    coords = list(wl.coords)
    masks = None if wl.isolated else masks
    # calibrate on a small prefix, then size the sample to the time budget
    k = min(len(coords), max(threads, 16))
    t = time.perf_counter()
    vox_oracle.baseline_run(cfg, coords[:k], None if masks is None else masks[:k], wl.index_base,
                            threads)
    per_chunk = max((time.perf_counter() - t) / k, 1e-7)
    sample = int(min(len(coords), max(threads, seconds / per_chunk / 4)))
    done, t0 = 0, time.perf_counter()
    passes = 0
    while True:
        vox_oracle.baseline_run(cfg, coords[:sample], None if masks is None else masks[:sample],
                                wl.index_base, threads)
        done += sample
        passes += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "chunks/s", "cores": threads, "kind": "port",
            "sample": f"{passes} passes over {sample} of {len(coords)} chunks of the same workload "
                      f"(Chunk::new + create_mesh per chunk, oracle restatement, {threads} threads)"}


def run_reference(args):
    """--impl reference: the reference's CPU chunk builder (the C restatement) on all host
    threads, on rank 0 only, for the same workload, metric and config as our arm."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    import voxgpu
    import vox_oracle
    wl = voxgpu.workload(args.workload)
    layout = voxgpu.LAYOUT_INSTANCED if args.layout == "instanced" else voxgpu.LAYOUT_VERTEX
    cfg = wl.config(layout=layout)
    masks = None if wl.isolated else wl.masks()
    threads = os.cpu_count() or 1
    coords = list(wl.coords)
    k = min(len(coords), 32)
    t = time.perf_counter()
    vox_oracle.baseline_run(cfg, coords[:k], None if masks is None else masks[:k], wl.index_base,
                            threads)
    per_chunk = max((time.perf_counter() - t) / k, 1e-7)
    budget = 90.0 / max(1, args.steps + args.warmup)  # the whole run within ~1.5 minutes
    sample = int(min(len(coords), max(1, budget / per_chunk)))
    # a step: passes over the sample for about a second (at most `budget`), so that every
    # step sees the same steady state as the in-run CPU baseline
    window = min(1.0, budget)

    def step():
        done, t0 = 0, time.perf_counter()
        while True:
            vox_oracle.baseline_run(cfg, coords[:sample], None if masks is None else masks[:sample],
                                    wl.index_base, threads)
            done += sample
            if time.perf_counter() - t0 >= window:
                return done, time.perf_counter() - t0
    for _ in range(args.warmup):
        step()
    results = [step() for _ in range(args.steps)]
    chunks = sum(d for d, _ in results)
    secs = sum(t for _, t in results)
    value = chunks / secs
    ms = 1e3 * sample / value  # time per pass over the sample
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "chunks/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32",
        "data": "synthetic",
        "config": config_of(args.workload, args.layout),
        "cpu_baseline": {"value": value, "unit": "chunks/s", "cores": threads, "kind": "port",
                         "sample": f"passes over {sample} of {len(coords)} chunks for about "
                                   f"{window:.1f} s per step; the reference is Rust (no toolchain "
                                   "here): its CPU chunk builder restated in C"},
        "e2e": {"value": value, "unit": "chunks/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def timed_steps(step, steps, stream, flush, torch, world=1):
    """Exactly `steps` calls of step(), L2 flushed before each (outside the events), CUDA
    events on the launching stream around each; returns (per-step ms, wall s)."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        torch.distributed.barrier()
    return [a.elapsed_time(b) for a, b in ev], wall


def measure_fused(name, args, torch, stream, flush, world=1, rank=0, local=0, headline=False):
    """One workload through the fused path: the whole batch resident, autotuned shape and
    slab, graph replays timed with events. Returns a dict of figures."""
    import voxgpu
    from voxgpu.batch import BatchRun
    wl = shard_workload(limited(voxgpu.workload(name), args.limit_chunks), rank, world)
    layout = voxgpu.LAYOUT_INSTANCED if args.layout == "instanced" else voxgpu.LAYOUT_VERTEX
    cfg = wl.config(layout=layout)
    masks = None if wl.isolated else wl.masks()
    ctx = voxgpu.Context(cfg, stream=stream.cuda_stream)
    if args.tuning:
        v = [int(x) for x in args.tuning.split(",")]
        ctx.set_tuning(*v)
    steps = args.steps if headline else (args.suite_steps or args.steps)
    with torch.cuda.stream(stream):
        run = BatchRun(ctx, wl.coords, masks, wl.index_base,
                       autotune=not (args.tuning or args.no_autotune), tune_iters=args.tune_iters,
                       graph=not args.no_graph)
    # nvidia-smi samples every 50 ms, longer than a short timed region: the sampler runs
    # from the warm-up, which keeps the GPU busy for about 0.3 s, through the timed steps
    sampler = ClockSampler(local).start()
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            run.launch()
        ctx.sync()
        t_hold = time.perf_counter()
        while time.perf_counter() - t_hold < args.clock_hold:
            for _ in range(8):
                run.launch()
            ctx.sync()
    step_ms, wall = timed_steps(run.launch, steps, stream, flush, torch, world)
    clocks = sampler.stop() | {"window": f"warm-up ({args.clock_hold:.1f} s of replays) through the "
                                         "timed steps"}
    st = ctx.sync(raise_on_error=False)
    assert st == voxgpu.VOX_OK, f"device status {st}"
    n = len(wl.coords)
    total = run.total_faces
    b0, b1 = run.b0, run.b1
    dev_ms = sum(step_ms)
    t = torch.tensor([dev_ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_per_step = float(t.item()) / steps
    peak, peak_kind = load_peak()
    launches = run.launches_per_step
    alg_bytes = total * (b0 + b1) + n * (12 + (0 if masks is None else 1)) + (n + 1) * 8
    kernel_ms = statistics.median(step_ms)
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    kname = {"phased": "k_mesh_batch_phased", "overlap": "k_mesh_batch_overlap"}.get(
        run.tuning.get("schedule"), "k_mesh_batch")
    staged = run.tuning.get("halo") == "pool"
    prof = NCU.get((kname + (" staged" if staged else ""), name))
    if staged:  # the step is the staged-halo sequence, the meshing kernel reading the pool
        kname += " (staged halo: coordinate map, neighbour lookup, k_generate into the pool)"
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "algorithmic_bytes_per_step": alg_bytes, "launches_per_step": launches,
            "timing": "median CUDA-event time of one step (all its launches), L2 flushed before "
                      "each step"}
    if prof and prof.get("per_step"):
        roof["traffic"] = prof["traffic"] * n / prof["chunks"]
        roof["traffic_source"] = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum summed over one "
                                  f"step's kernels ({prof['summary']}), per step like achieved")
    elif prof:
        per_launch_chunks = n / launches
        roof["traffic"] = prof["traffic"] * per_launch_chunks / prof["chunks"]
        roof["traffic_source"] = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch "
                                  f"({prof['summary']})"
                                  + (f", captured on {prof['scaled_from_chunks']} chunks and scaled "
                                     "by the chunk count" if "scaled_from_chunks" in prof else "")
                                  + ("" if per_launch_chunks == prof["chunks"]
                                     else f", scaled from {prof['chunks']} to {per_launch_chunks:.0f} "
                                          "chunks per launch"))
    else:
        roof["traffic"] = None
    res = {"value": n * world / (ms_per_step / 1e3), "unit": "chunks/s", "ms_per_step": ms_per_step,
           "steps": steps, "chunks": n, "voxels_per_s": n * world / (ms_per_step / 1e3) * cfg.chunk_size ** 3,
           "faces_per_step": total, "launches_per_step": launches, "tuning": run.tuning,
           "launch": ("vox_gen_mesh_batch" if args.no_graph
                      else "CUDA graph replay (one captured graph holding every slab launch)"),
           "l2": "flushed before every step (256 MiB write, outside the events)",
           "roofline": roof, "clocks": clocks, "wall_s_timed_region": wall,
           "gpu_launches": steps * launches}
    if prof and "warp_instructions" in prof and launches == 1:
        instr = prof["warp_instructions"] * n / prof["chunks"]
        res["issue_roofline"] = {
            "warp_instructions_per_launch": instr, "achieved": instr / (kernel_ms / 1e3),
            "peak": ISSUE_PEAK, "unit": "warp instructions/s",
            "frac": instr / (kernel_ms / 1e3) / ISSUE_PEAK,
            "peak_source": "nominal (152 SMs x 4 schedulers x 2.07 GHz); instructions from "
                           + prof["summary"]}
    # with staged halos no halo sample is evaluated (every neighbour of these workloads is in
    # the batch and is read from the pool)
    noise = noise_report(wl, cfg, masks if masks is not None and not staged else [0] * n,
                         ms_per_step)
    if noise:
        res["noise_fp32"] = noise
    extras = {"wl": wl, "cfg": cfg, "masks": masks, "ctx": ctx, "run": run}
    return res, extras


def plain_per_chunk(ctx, wl, cfg, masks, stream, args, torch, limit):
    """Chunk::new then create_mesh per chunk, one launch each (no batching), for the first
    `limit` chunks of the workload: every generate and mesh launch is captured once into a
    CUDA graph and the graph is replayed, so the time is the GPU's alone. Chunks whose
    occupancy those meshes read as a neighbour are generated too."""
    n = len(wl.coords)
    k = min(n, limit)
    words = ctx.sizes.occ_words_per_chunk
    per = ctx.sizes.max_faces_per_chunk
    b0, b1 = ctx.sizes.bytes_per_face_out0, ctx.sizes.bytes_per_face_out1
    occ = torch.empty(n * words, dtype=torch.int32, device="cuda")
    o0 = torch.empty(k * per * b0, dtype=torch.uint8, device="cuda")
    o1 = torch.empty(k * per * b1, dtype=torch.uint8, device="cuda") if b1 else None
    cnt = torch.zeros(k, dtype=torch.int64, device="cuda")
    d_coords = torch.tensor(list(wl.coords), dtype=torch.int32, device="cuda")
    index = {c: i for i, c in enumerate(wl.coords)}
    offs = [(-1, 0, 0), (1, 0, 0), (0, 0, -1), (0, 0, 1), (0, -1, 0), (0, 1, 0)]
    occp, cp = occ.data_ptr(), d_coords.data_ptr()
    o0p, o1p = o0.data_ptr(), (o1.data_ptr() if o1 is not None else 0)
    gen, meshes = set(range(k)), []
    for i in range(k):
        c = wl.coords[i]
        nb = []
        for d, (dx, dy, dz) in enumerate(offs):
            j = index.get((c[0] + dx, c[1] + dy, c[2] + dz))
            ok = masks is not None and (masks[i] >> d) & 1 and j is not None
            if ok:
                gen.add(j)
            nb.append(occp + 4 * words * j if ok else None)
        meshes.append((occp + 4 * words * i, nb, c, o0p + i * per * b0,
                       (o1p + i * per * b1) if b1 else None, cnt.data_ptr() + 8 * i))
    gen = sorted(gen)

    def one_pass():
        for i in gen:
            ctx.generate(cp + 12 * i, 1, occp + 4 * words * i, chunk_index_base=wl.index_base + i)
        for (self_p, nb, c, p0, p1, cntp) in meshes:
            ctx.mesh(self_p, nb, c, p0, p1, per, cntp)

    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        one_pass()  # direct launches once (warms the kernels up)
    ctx.sync()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        g.capture_begin()
        one_pass()
        g.capture_end()
        g.replay()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.plain_steps):
            g.replay()
        t1.record(stream)
        torch.cuda.synchronize()
    assert ctx.sync(raise_on_error=False) == 0
    ms = t0.elapsed_time(t1) / args.plain_steps
    del g
    return {"value": k / (ms / 1e3), "unit": "chunks/s", "chunks_per_pass": k,
            "generate_launches": len(gen), "mesh_launches": k, "ms_per_pass": ms,
            "api": "vox_generate + vox_mesh per chunk, one launch each, captured once as a CUDA "
                   "graph and replayed (GPU time only, no host dispatch in the events)"}


def noise_kernel(ctx, wl, cfg, stream, flush, args, torch):
    """The generation kernel alone (Chunk::new, src/chunk.rs:21-46): vox_generate writes the
    occupancy of every chunk (no halo) to a device pool; its noise FP32 work is samples x
    octaves x the formula's operation count, against the nominal FP32 instruction rate."""
    g = cfg.gen
    if g.kind not in (0, 1):
        return None
    n = len(wl.coords)
    N = cfg.chunk_size
    samples, dim = (N * N, 2) if g.kind == 0 else (N ** 3, 3)
    d_coords = torch.tensor(list(wl.coords), dtype=torch.int32, device="cuda")
    pool = torch.empty(n * ctx.sizes.occ_words_per_chunk, dtype=torch.int32, device="cuda")
    steps = max(3, (args.suite_steps or args.steps) // 4)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for _ in range(3):
            ctx.generate(d_coords, n, pool, chunk_index_base=wl.index_base)
    step_ms, _ = timed_steps(lambda: ctx.generate(d_coords, n, pool, chunk_index_base=wl.index_base),
                             steps, stream, flush, torch)
    assert ctx.sync(raise_on_error=False) == 0
    ms = statistics.median(step_ms)
    ops = n * samples * g.octaves * own_noise_ops(cfg)
    achieved = ops / (ms / 1e3)
    return {"kernel": "k_generate", "ms": ms, "steps": steps, "chunks": n,
            "samples_per_chunk": samples, "octaves": g.octaves,
            "exec_ops_per_sample_octave": own_noise_ops(cfg),
            "formula_ops_per_sample_octave": NOISE_OPS[dim], "achieved_tops": achieved / 1e12,
            "peak_tops": FP32_OPS_NOMINAL / 1e12, "peak_source": FP32_PEAK_SOURCE,
            "frac": achieved / FP32_OPS_NOMINAL,
            "formula_tops": n * samples * g.octaves * NOISE_OPS[dim] / (ms / 1e3) / 1e12,
            "occupancy_bytes": n * ctx.sizes.occ_words_per_chunk * 4,
            "bound": ("FP32 pipe (FMA pipe 64 % active under ncu, math_pipe_throttle the top stall: "
                      "profiles/k_generate_density.md)" if g.kind == 1 else
                      "latency: one wave of one-chunk CTAs, each evaluating its columns' fBm as "
                      "chains of dependent permutation-table reads and writing 1 KiB; the FP32 "
                      "fraction is not this kernel's bound"),
            "api": "vox_generate (occupancy to a device pool, L2 flushed before each step)"}


def mesh_from_occupancy(ctx, wl, run, stream, flush, args, torch):
    """The rebuild path (ChunkGenerator::process_rebuild_queue, src/chunk_builder.rs:89-112):
    vox_mesh_batch over occupancy already resident in a device pool (filled once by
    vox_generate, untimed), with the lateral neighbours' slots as the halo source. Its output
    must equal the fused path's byte for byte."""
    import numpy as np
    n = run.n
    words = ctx.sizes.occ_words_per_chunk
    pool = torch.empty(n * words, dtype=torch.int32, device="cuda")
    index = {tuple(c): i for i, c in enumerate(wl.coords)}
    nbr = np.full((n, 6), -1, np.int32)
    for i, (x, y, z) in enumerate(wl.coords):
        for d, (dx, dz) in enumerate(((-1, 0), (1, 0), (0, -1), (0, 1))):
            nbr[i, d] = index.get((x + dx, y, z + dz), -1)
    d_slots = torch.arange(n, dtype=torch.int32, device="cuda")
    d_nbr = torch.from_numpy(nbr).cuda()
    offs = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    total = run.total_faces
    want0 = run.out0[:total * run.b0].clone()
    want1 = run.out1[:total * run.b1].clone() if run.b1 else None
    o0 = torch.empty_like(run.out0)
    o1 = torch.empty_like(run.out1) if run.out1 is not None else None
    steps = max(3, (args.suite_steps or args.steps) // 4)
    torch.cuda.synchronize()  # the buffers above were filled on the default stream
    with torch.cuda.stream(stream):
        ctx.generate(run.d_coords, n, pool, chunk_index_base=wl.index_base)
        for _ in range(3):
            ctx.mesh_batch(pool, n, d_slots, d_nbr, run.d_coords, n, o0, o1, run.cap, offs)
    step_ms, _ = timed_steps(
        lambda: ctx.mesh_batch(pool, n, d_slots, d_nbr, run.d_coords, n, o0, o1, run.cap, offs),
        steps, stream, flush, torch)
    assert ctx.sync(raise_on_error=False) == 0
    same = (torch.equal(offs, run.offsets) and torch.equal(o0[:total * run.b0], want0)
            and (want1 is None or torch.equal(o1[:total * run.b1], want1)))
    assert same, "the rebuild path must write the fused path's bytes"
    ms = statistics.median(step_ms)
    return {"value": n / (ms / 1e3), "unit": "chunks/s", "ms_per_step": ms, "steps": steps,
            "bytes_equal_to_fused": True,
            "api": "vox_mesh_batch from device-resident occupancy (L2 flushed before each step)"}


def e2e_host(ctx, wl, masks, n, total_faces, b0, b1, args):
    """vox_gen_mesh_host with pinned host buffers: the coordinates and neighbour masks
    come from host memory and every emitted face and offset lands in host memory, all
    inside the timed call (the kernel reads and writes the page-locked buffers in place)."""
    import ctypes

    import numpy as np

    import voxgpu
    L = voxgpu.lib()

    def pinned(nbytes):
        p = ctypes.c_void_p()
        assert L.vox_host_alloc(max(16, nbytes), ctypes.byref(p)) == 0
        return p.value

    h_coords = pinned(n * 12)
    h_mask = pinned(n) if masks is not None else None
    ctypes.memmove(h_coords, np.asarray(wl.coords[:n], np.int32).tobytes(), n * 12)
    if masks is not None:
        ctypes.memmove(h_mask, np.asarray(masks[:n], np.uint8).tobytes(), n)
    h0 = pinned(total_faces * b0)
    h1 = pinned(total_faces * b1) if b1 else None
    h_offs = pinned((n + 1) * 8)
    for _ in range(3):
        ctx.gen_mesh_host(h_coords, h_mask, n, h0, h1, total_faces, h_offs,
                          chunk_index_base=wl.index_base)
    times = []
    for _ in range(args.e2e_steps):
        t = time.perf_counter()
        ctx.gen_mesh_host(h_coords, h_mask, n, h0, h1, total_faces, h_offs,
                          chunk_index_base=wl.index_base)
        times.append(time.perf_counter() - t)
    for p in (h_coords, h_mask, h0, h1, h_offs):
        if p:
            L.vox_host_free(p)
    ms = 1e3 * statistics.median(times)
    h2d = n * (12 + (1 if masks is not None else 0))
    d2h = (n + 1) * 8 + total_faces * (b0 + b1)
    return {"value": n / (ms / 1e3), "unit": "chunks/s", "ms_per_step": ms,
            "host_link_gbs": (h2d + d2h) / (ms / 1e3) / 1e9,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "api": "vox_gen_mesh_host (pinned host buffers: the kernel reads the inputs and "
                   "writes faces and offsets in host memory over NVLink-C2C; synchronous)"}


def serving_run(frames: int, paced: bool, view_radius: int = 24, slots: int = 4,
                max_batch: int = 256):
    """The serving workload: the simulated camera (20 units/s along +x, 90 deg/s yaw
    sweep, 60 frames/s) drives the streaming engine over the heightmap terrain (16^3
    chunks, view radius 24 chunks, 24 GB device cache with LRU eviction). Paced: frame k
    starts at k/60 s of wall time; unpaced: frames back to back (maximum request rate)."""
    import voxgpu
    wl = voxgpu.workload("heightmap")
    srv = voxgpu.Server(wl.config(), view_radius=view_radius, max_batch=max_batch, slots=slots,
                        cache_budget_bytes=24 << 30)
    zfar = (view_radius + 2) * 16.0
    t0 = voxgpu.Server.now()
    late = 0
    for k in range(frames):
        ts = k / 60.0
        if paced:
            while voxgpu.Server.now() - t0 < ts:
                time.sleep(0.0005)
            late = max(late, voxgpu.Server.now() - t0 - ts)
        eye, d = voxgpu.serving_camera(ts)
        srv.frame(voxgpu.camera_matrix(eye, d, zfar=zfar), eye)
    srv.drain()
    wall = voxgpu.Server.now() - t0
    st = srv.stats()
    steady = srv.latency(t0 + 1.0)
    srv.close()
    return {
        "frames": frames, "paced_60fps": paced, "requested": st.requested,
        "completed": st.completed, "launches": st.launches, "evicted": st.evicted,
        "chunks_per_launch": st.completed / st.launches if st.launches else None,
        "p50_ms": st.latency_p50_ms, "p99_ms": st.latency_p99_ms, "max_ms": st.latency_max_ms,
        "steady_state": {"after_s": 1.0, "requests": steady[3], "p50_ms": steady[0],
                         "p99_ms": steady[1], "max_ms": steady[2],
                         "note": "requests issued after the first second (the first frame's "
                                 "view-disk fill excluded)"},
        "request_rate_chunks_per_s": st.completed / wall if wall > 0 else None,
        "wall_s": wall, "frame_budget_ms": 1000.0 / 60,
        "max_frame_start_lag_ms": 1e3 * late if paced else None,
    }


def serving_capacity(chunks: int, max_batch: int = 1024, slots: int = 4):
    """Unpaced capacity of the streaming engine: `chunks` requests of the serving terrain
    (a square of 16^3 chunks) submitted at once and drained; chunks/s from the first request
    to the last completion (continuous batching over `slots` streams, `max_batch` chunks per
    launch)."""
    import voxgpu
    wl = voxgpu.workload("heightmap")
    side = int(round(chunks ** 0.5))
    coords = [(x, 0, z) for z in range(-side // 2, side - side // 2)
              for x in range(-side // 2, side - side // 2)]
    srv = voxgpu.Server(wl.config(), view_radius=24, max_batch=max_batch, slots=slots,
                        cache_budget_bytes=24 << 30)
    warm = [(x, 0, 10_000) for x in range(max_batch)]
    srv.submit(warm)
    srv.drain()
    srv.close()
    srv = voxgpu.Server(wl.config(), view_radius=24, max_batch=max_batch, slots=slots,
                        cache_budget_bytes=24 << 30)
    t0 = voxgpu.Server.now()
    srv.submit(coords, now=t0)
    srv.drain()
    wall = voxgpu.Server.now() - t0
    st = srv.stats()
    srv.close()
    return {"chunks": len(coords), "completed": st.completed, "launches": st.launches,
            "chunks_per_launch": st.completed / st.launches if st.launches else None,
            "max_batch": max_batch, "slots": slots, "busy_s": st.busy_s, "wall_s": wall,
            "chunks_per_s": st.completed / st.busy_s if st.busy_s > 0 else None,
            "p50_ms": st.latency_p50_ms, "p99_ms": st.latency_p99_ms,
            "api": "vox_serve_submit of every chunk at once, then vox_serve_drain"}


def sub_workload(name, args, torch, stream, flush, e2e_chunks=None, cpu_seconds=4.0,
                 plain_limit=0):
    """A suite entry: the fused path's figures, its end-to-end call, the plain per-chunk GPU
    path on a prefix and the CPU port on a sample."""
    res, ex = measure_fused(name, args, torch, stream, flush)
    wl, cfg, masks, ctx, run = ex["wl"], ex["cfg"], ex["masks"], ex["ctx"], ex["run"]
    res["config"] = config_of(name, args.layout, args.limit_chunks)
    if plain_limit and args.plain_steps > 0:
        res["plain_per_chunk"] = plain_per_chunk(ctx, wl, cfg, masks, stream, args, torch,
                                                 plain_limit)
        res["batched_vs_plain"] = res["value"] / res["plain_per_chunk"]["value"]
    if name == "density":
        res["noise_kernel"] = noise_kernel(ctx, wl, cfg, stream, flush, args, torch)
    n = len(wl.coords)
    n_e2e = min(n, e2e_chunks or n)
    faces = run.total_faces if n_e2e == n else int(run.offsets[n_e2e].item())
    run.close()
    torch.cuda.empty_cache()
    res["e2e"] = e2e_host(ctx, wl, masks, n_e2e, faces, run.b0, run.b1, args)
    if n_e2e < n:
        res["e2e"]["sample"] = f"first {n_e2e} of {n} chunks"
    if not args.no_cpu:
        res["cpu_baseline"] = cpu_baseline(wl, cfg, masks, cpu_seconds)
    ctx.close()
    torch.cuda.empty_cache()
    return res


def run_ours(args):
    """Our arm: the workload's batch on this rank's GPU (graph replays, L2 flushed), with
    e2e, roofline, CPU baseline and, by default, the stress, density and serving sub-runs."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    res, ex = measure_fused(args.workload, args, torch, stream, flush, world, rank, local,
                            headline=True)
    wl, cfg, masks, ctx, run = ex["wl"], ex["cfg"], ex["masks"], ex["ctx"], ex["run"]
    if rank == 0:
        print(f"launch shape: {res['tuning']}", file=sys.stderr, flush=True)
    line = {
        "metric": METRIC, "value": res["value"], "unit": "chunks/s", "n_gpus": world,
        "steps": res["steps"], "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32",
        "data": "synthetic",
        "config": config_of(args.workload, args.layout, args.limit_chunks),
        "launch": {k: res[k] for k in ("tuning", "launches_per_step", "faces_per_step", "launch",
                                       "l2")} | {"parallelism": f"dp{world} (independent chunk "
                                                                "batches, no exchange)"},
        "voxels_per_s": res["voxels_per_s"],
        "roofline": res["roofline"],
        "gpu_launches": res["gpu_launches"],
        "wall_s_timed_region": res["wall_s_timed_region"],
        "clocks": res["clocks"],
    }
    for k in ("issue_roofline", "noise_fp32"):
        if k in res:
            line[k] = res[k]
    if rank == 0:
        n = len(wl.coords)
        if args.plain_steps > 0:
            limit = {8: 1024, 16: 1024, 32: 256}.get(cfg.chunk_size, 32)
            line["plain_per_chunk"] = plain_per_chunk(ctx, wl, cfg, masks, stream, args, torch, limit)
            line["batched_vs_plain"] = res["value"] / world / line["plain_per_chunk"]["value"]
        if not wl.isolated and run.launches_per_step >= 1 and cfg.chunk_size <= 32:
            line["mesh_from_occupancy"] = mesh_from_occupancy(ctx, wl, run, stream, flush, args, torch)
        if cfg.gen.kind in (0, 1):
            line["noise_kernel"] = noise_kernel(ctx, wl, cfg, stream, flush, args, torch)
        n_e2e = min(n, 64) if args.workload == "stress" else n
        faces = run.total_faces if n_e2e == n else int(run.offsets[n_e2e].item())
        b0, b1 = run.b0, run.b1
        run.close()
        torch.cuda.empty_cache()
        line["e2e"] = e2e_host(ctx, wl, masks, n_e2e, faces, b0, b1, args)
        if n_e2e < n:
            line["e2e"]["sample"] = f"first {n_e2e} of {n} chunks"
        if world == 1 and not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(wl, cfg, masks, args.cpu_seconds * 0.75)
            line["cpu_baseline_single_thread"] = cpu_baseline(wl, cfg, masks,
                                                              args.cpu_seconds * 0.25, threads=1)
    else:
        run.close()
    ctx.close()
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and args.workload == "heightmap" and not args.no_suite:
        # the other workloads of the suite, each with its own timed region and clocks
        line["stress"] = sub_workload("stress", args, torch, stream, flush, e2e_chunks=64,
                                      plain_limit=32)
        line["density"] = sub_workload("density", args, torch, stream, flush, plain_limit=256)
        del flush
        torch.cuda.empty_cache()
        serving = {"workload": SERVING_TEXT}
        if args.capacity_chunks > 0:
            serving["capacity"] = serving_capacity(args.capacity_chunks)
        if args.serving_frames > 0:
            serving["paced"] = serving_run(args.serving_frames, paced=True)
        line["serving"] = serving
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_serving(args):
    """--workload serving: the streaming engine alone (paced frames and capacity)."""
    rank, world, local = dist_info()
    import torch
    torch.cuda.set_device(local)
    frames = args.frames
    res = serving_run(frames, args.paced)
    line = {
        "metric": METRIC, "value": res["request_rate_chunks_per_s"], "unit": "chunks/s",
        "n_gpus": 1, "steps": frames, "warmup": 0, "ms_per_step": res["wall_s"] * 1e3 / frames,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32",
        "data": "synthetic",
        "config": {"workload": SERVING_TEXT, "paced": args.paced},
        "latency": res,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    """Dispatches to the reference arm, the serving run or our arm."""
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
