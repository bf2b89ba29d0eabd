#!/usr/bin/env python3
"""Benchmark of the chunk generation + meshing path (one JSON line on stdout).

Default workload: 32x32 = 1024 chunks of 16^3 with a 2-D fBm heightmap (4 octaves,
lacunarity 2, gain 0.5, f = 1/128, seed 7, amplitude 48, base 8), meshed in the
vertex layout (4 x 24-byte vertices + 6 u32 indices per face). One step = one fused
generation + meshing launch over the whole batch (vox_gen_mesh_batch). The same batch
is also run through the plain per-chunk path (one generate + one mesh launch per
chunk) and end to end through the host-pointer entry point (vox_gen_mesh_host, pinned
host buffers, copies inside the timed region).

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
              "vertex layout, launched in slabs of --slab chunks",
}
L2_FLUSH_BYTES = 256 << 20


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=400)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=list(WORKLOAD_TEXT) + ["serving"], default="heightmap")
    p.add_argument("--layout", choices=["vertex", "instanced"], default="vertex")
    p.add_argument("--slab", type=int, default=1024,
                   help="chunks per launch (stress workload; 1024 x 48 MB of output per launch)")
    p.add_argument("--cpu-seconds", type=float, default=8.0,
                   help="wall time of the CPU-baseline sample")
    p.add_argument("--e2e-steps", type=int, default=50)
    p.add_argument("--plain-steps", type=int, default=3)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--no-graph", action="store_true",
                   help="launch through vox_gen_mesh_batch instead of replaying captured graphs")
    p.add_argument("--tuning", default=None,
                   help="force a launch shape 'threads,stage_faces,ctas_per_sm[,schedule]' "
                        "(schedule 0 look-back, 1 phased, 2 overlap; no autotune)")
    p.add_argument("--frames", type=int, default=10000, help="serving workload: frames")
    p.add_argument("--paced", action="store_true", help="serving workload: real-time 60 fps")
    p.add_argument("--latency-frames", type=int, default=300,
                   help="paced serving frames measured for the headline latency (0: skip)")
    p.add_argument("--tune-iters", type=int, default=5)
    return p.parse_args()


def dist_info():
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
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_value(kernel: str, workload: str, key: str = "traffic_bytes_per_launch"):
    """A per-launch figure recorded from an ncu capture in profiles/ (or None)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per launch recorded from an ncu capture in profiles/ (or None)."""
    return profiled_value(kernel, workload)


# Warp-instruction issue capacity: 152 SMs x 4 schedulers x 2.07 GHz (nominal).
ISSUE_PEAK = 152 * 4 * 2.07e9


# FP32 operations of one noise sample-octave in the noise formula (the oracle's
# or_noise2_f32 / or_noise3_f32 plus one fBm step): floors, fractional parts, fades
# (7 each), corner gradients (2-D: 2 mul + 1 add; 3-D: 3 mul + 2 add), lerps (3 each),
# the coordinate scaling and the fBm update (sum, amp, f).
NOISE_OPS = {2: 2 + 2 + 14 + 2 + 4 * 3 + 3 * 3 + 2 + 4, 3: 3 + 3 + 21 + 3 + 8 * 5 + 7 * 3 + 3 + 4}
# FP32 instruction rate with FMA contraction off (one op per instruction): 152 SMs x 128
# lanes x 2.07 GHz. Nominal: the measured peaks file has no FP32 figure.
FP32_OPS_NOMINAL = 152 * 128 * 2.07e9


def noise_report(wl, cfg, masks, ms_per_step):
    """Algorithmic FP32 throughput of the noise in one step: samples x octaves x ops."""
    N = cfg.chunk_size
    g = cfg.gen
    n_chunks = len(masks)
    if g.kind == 0:    # heightmap: 2-D noise per column, (N + 2)^2 - 4 columns with halo
        samples, dim = (N + 2) ** 2 - 4, 2
        total = n_chunks * samples
    elif g.kind == 1:  # density: 3-D noise per voxel and per halo voxel of a loaded neighbour
        samples, dim = N ** 3, 3
        used = 0x3F if cfg.cull_mode == 1 else 0x0F
        total = n_chunks * samples + sum(bin(m & used).count("1") for m in masks) * N * N
        samples = total / n_chunks
    else:
        return None
    ops = total * g.octaves * NOISE_OPS[dim]
    achieved = ops / (ms_per_step / 1e3)
    return {"samples_per_chunk": samples, "octaves": g.octaves, "ops_per_sample_octave": NOISE_OPS[dim],
            "achieved_tops": achieved / 1e12, "peak_tops": FP32_OPS_NOMINAL / 1e12,
            "peak_source": "nominal FP32 instruction rate (FMA contraction off)",
            "frac": achieved / FP32_OPS_NOMINAL,
            "note": "the fused launch also culls and emits; this is the noise share of the step's "
                    "time budget, not the noise kernel alone"}


def cpu_baseline(wl, cfg, masks, seconds: float, threads: int = 0):
    """The oracle restatement of the reference CPU chunk builder on `threads` host threads
    (0: all), repeated over the workload (or a prefix of it) for about `seconds`."""
    import vox_oracle
    threads = threads or os.cpu_count() or 1
    coords = list(wl.coords)
    # calibrate on a small prefix, then size the sample to the time budget
    k = min(len(coords), 64)
    t = time.perf_counter()
    vox_oracle.baseline_run(cfg, coords[:k], masks[:k], wl.index_base, threads)
    per_chunk = max((time.perf_counter() - t) / k, 1e-7)
    sample = int(min(len(coords), max(8, seconds / per_chunk / 4)))
    done, t0 = 0, time.perf_counter()
    passes = 0
    while True:
        vox_oracle.baseline_run(cfg, coords[:sample], masks[:sample], wl.index_base, threads)
        done += sample
        passes += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "chunks/s", "cores": threads, "kind": "port",
            "sample": f"{passes} passes over {sample} of {len(coords)} chunks of the same workload "
                      f"(Chunk::new + create_mesh per chunk, oracle restatement, {threads} threads)"}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    import voxgpu
    import vox_oracle
    wl = voxgpu.workload(args.workload)
    layout = voxgpu.LAYOUT_INSTANCED if args.layout == "instanced" else voxgpu.LAYOUT_VERTEX
    cfg = wl.config(layout=layout)
    masks = wl.masks()
    threads = os.cpu_count() or 1
    coords = list(wl.coords)
    k = min(len(coords), 32)
    t = time.perf_counter()
    vox_oracle.baseline_run(cfg, coords[:k], masks[:k], wl.index_base, threads)
    per_chunk = max((time.perf_counter() - t) / k, 1e-7)
    budget = 90.0 / max(1, args.steps + args.warmup)  # the whole run within ~1.5 minutes
    sample = int(min(len(coords), max(1, budget / per_chunk)))
    # a step: passes over the sample for about a second (at most `budget`), so that every
    # step sees the same steady state as the in-run CPU baseline
    window = min(1.0, budget)

    def step():
        done, t0 = 0, time.perf_counter()
        while True:
            vox_oracle.baseline_run(cfg, coords[:sample], masks[:sample], wl.index_base, threads)
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
        "config": {"workload": WORKLOAD_TEXT[args.workload], "chunks": len(coords),
                   "chunk_size": cfg.chunk_size, "layout": args.layout,
                   "chunks_per_step": sample},
        "cpu_baseline": {"value": value, "unit": "chunks/s", "cores": threads, "kind": "port",
                         "sample": f"passes over {sample} of {len(coords)} chunks for about "
                                   f"{window:.1f} s per step; the reference is Rust (no toolchain "
                                   "here): its CPU chunk builder restated in C"},
        "e2e": {"value": value, "unit": "chunks/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    import voxgpu

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl = shard_workload(voxgpu.workload(args.workload), rank, world)
    layout = voxgpu.LAYOUT_INSTANCED if args.layout == "instanced" else voxgpu.LAYOUT_VERTEX
    cfg = wl.config(layout=layout)
    masks = wl.masks()
    n_all = len(wl.coords)
    stream = torch.cuda.Stream()
    ctx = voxgpu.Context(cfg, stream=stream.cuda_stream)
    b0, b1 = ctx.sizes.bytes_per_face_out0, ctx.sizes.bytes_per_face_out1
    slab = args.slab if args.workload == "stress" else n_all
    slabs = [(s, min(n_all, s + slab)) for s in range(0, n_all, slab)]
    d_coords = torch.tensor(wl.coords, dtype=torch.int32, device="cuda")
    d_mask = torch.tensor(masks, dtype=torch.uint8, device="cuda")
    d_offs = torch.zeros(n_all + len(slabs), dtype=torch.int64, device="cuda")

    # size the output from one sizing pass (the output is deterministic)
    max_slab_faces = 0
    with torch.cuda.stream(stream):
        probe_cap = 0
        for si, (a, b) in enumerate(slabs):
            offs = d_offs[a + si:b + si + 1]
            ctx.gen_mesh_batch(d_coords[a:b], d_mask[a:b], b - a, None, None, probe_cap, offs,
                               chunk_index_base=wl.index_base + a)
            ctx.sync(raise_on_error=False)
            max_slab_faces = max(max_slab_faces, int(offs[-1].item()))
    cap = max_slab_faces
    o0 = torch.empty(cap * b0 + 16, dtype=torch.uint8, device="cuda")
    o1 = torch.empty(cap * b1 + 16, dtype=torch.uint8, device="cuda") if b1 else None
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    total_faces = 0
    # launch shape from the autotuner, timed on the first slab (setup, not timed)
    tuning = None
    if args.tuning:
        ctx.set_tuning(*(int(v) for v in args.tuning.split(",")))
    elif not args.no_autotune:
        a, b = slabs[0]
        with torch.cuda.stream(stream):
            tuning = ctx.autotune(d_coords[a:b], d_mask[a:b], b - a, o0, o1, cap, d_offs[a:b + 1],
                                  chunk_index_base=wl.index_base + a, iters=args.tune_iters)
    tuning = ctx.tuning().as_dict() | {"autotuned": tuning is not None}
    if rank == 0:
        print(f"launch shape: {tuning}", file=sys.stderr, flush=True)

    # each slab's launch captured once as a CUDA graph and replayed every step
    graphs = []
    if not args.no_graph:
        with torch.cuda.stream(stream):
            for si, (a, b) in enumerate(slabs):
                graphs.append(ctx.capture_graph(d_coords[a:b], d_mask[a:b], b - a, o0, o1, cap,
                                                d_offs[a + si:b + si + 1],
                                                chunk_index_base=wl.index_base + a))

    def step():
        if graphs:
            for g in graphs:
                g.launch()
            return
        for si, (a, b) in enumerate(slabs):
            ctx.gen_mesh_batch(d_coords[a:b], d_mask[a:b], b - a, o0, o1, cap,
                               d_offs[a + si:b + si + 1], chunk_index_base=wl.index_base + a)

    sampler = ClockSampler(local)
    sampler.start()
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        ctx.sync()
        for si, (a, b) in enumerate(slabs):
            total_faces += int(d_offs[b + si].item())
        # timed region: exactly K steps, L2 flushed before each, CUDA events on the
        # launching stream around each step
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        st = ctx.sync(raise_on_error=False)
        assert st == voxgpu.VOX_OK, f"device status {st}"
        if world > 1:
            torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_ms = sum(step_ms)
    t = torch.tensor([dev_ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    max_ms = float(t.item())
    ms_per_step = max_ms / args.steps
    chunks_all = n_all * world
    value = chunks_all / (ms_per_step / 1e3)

    # plain per-chunk path: one generate + one mesh launch per chunk
    plain = None
    if rank == 0 and args.plain_steps > 0:
        plain = plain_per_chunk(ctx, wl, cfg, d_coords, stream, args, b0, b1, torch, np)

    # the rebuild path: meshing from resident occupancy (workloads with neighbours)
    rebuild = None
    if rank == 0 and len(slabs) == 1 and not wl.isolated:
        rebuild = mesh_from_occupancy(ctx, wl, cfg, d_coords, n_all, o0, o1, cap, total_faces,
                                      stream, flush, args, torch, np)
    # the generation kernel alone (heightmap and density generators)
    gen_alone = None
    if rank == 0 and len(slabs) == 1:
        gen_alone = noise_kernel(ctx, wl, cfg, d_coords, n_all, stream, flush, args, torch)
    # end to end through the host-pointer entry point (pinned buffers); the stress output
    # (49 GB per 1024 chunks) is sampled on its first 64 chunks
    e2e = None
    if rank == 0:
        # (within the first slab, whose offsets start at d_offs[0])
        n_e2e = min(slabs[0][1], 64) if args.workload == "stress" else n_all
        faces_e2e = total_faces if n_e2e == n_all and len(slabs) == 1 else int(d_offs[n_e2e].item())
        e2e = e2e_host(ctx, wl, masks, n_e2e, faces_e2e, b0, b1, args, np)
        if n_e2e < n_all:
            e2e["sample"] = f"first {n_e2e} of {n_all} chunks"
    clocks = sampler.stop()

    peak, peak_kind = load_peak()
    alg_bytes = total_faces * (b0 + b1) + n_all * (12 + 1) + (n_all + len(slabs)) * 8
    kernel_ms = statistics.median(step_ms)
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    kname = {"phased": "k_mesh_batch_phased", "overlap": "k_mesh_batch_overlap"}.get(
        tuning.get("schedule"), "k_mesh_batch")
    traffic = profiled_traffic(kname, args.workload)
    line = {
        "metric": METRIC, "value": value, "unit": "chunks/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD_TEXT[args.workload], "chunks": n_all,
                   "chunk_size": cfg.chunk_size, "layout": args.layout,
                   "faces_per_step": total_faces, "launches_per_step": len(slabs),
                   "launch": ("vox_gen_mesh_batch" if args.no_graph
                              else "CUDA graph replay (one captured graph per slab)"),
                   "tuning": tuning,
                   "l2": "flushed before every step (256 MiB write, outside the events)",
                   "parallelism": f"dp{world} (independent chunk batches)"},
        "voxels_per_s": value * cfg.chunk_size ** 3,
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes / len(slabs),
                     "traffic": traffic},
        "gpu_launches": args.steps * len(slabs),
        "wall_s_timed_region": wall,
        "clocks": clocks,
    }
    if plain:
        line["plain_per_chunk"] = plain
        line["batched_vs_plain"] = value / world / plain["value"]
    if e2e:
        line["e2e"] = e2e
    if rebuild:
        line["mesh_from_occupancy"] = rebuild
    if gen_alone:
        line["noise_kernel"] = gen_alone
    if rank == 0 and world == 1 and args.latency_frames > 0 and args.workload == "heightmap":
        # p50/p99 request-to-mesh latency of the streaming engine at the serving request
        # rate (real-time 60 frames/s camera), next to the batch throughput above
        line["latency"] = serving_run(args.latency_frames, paced=True)
    instr = profiled_value(kname, args.workload, "warp_instructions_per_launch")
    if instr and len(slabs) == 1:
        # the same launch against the warp-instruction issue rate: for a launch whose
        # output stays in L2 this, not HBM, is the budget it spends
        line["issue_roofline"] = {
            "warp_instructions_per_launch": instr, "achieved": instr / (kernel_ms / 1e3),
            "peak": ISSUE_PEAK, "unit": "warp instructions/s", "frac": instr / (kernel_ms / 1e3) / ISSUE_PEAK,
            "peak_source": "nominal (152 SMs x 4 schedulers x 2.07 GHz); instructions from the ncu "
                           "capture in profiles/"}
    noise = noise_report(wl, cfg, masks, ms_per_step)
    if noise:
        line["noise_fp32"] = noise
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(wl, cfg, masks, args.cpu_seconds * 0.75)
        line["cpu_baseline_single_thread"] = cpu_baseline(wl, cfg, masks, args.cpu_seconds * 0.25,
                                                          threads=1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def plain_per_chunk(ctx, wl, cfg, d_coords, stream, args, b0, b1, torch, np):
    """Chunk::new then create_mesh per chunk, one launch each (no batching)."""
    n = len(wl.coords)
    words = ctx.sizes.occ_words_per_chunk
    occ = torch.empty(n * words, dtype=torch.int32, device="cuda")
    per = ctx.sizes.max_faces_per_chunk
    k = min(n, 256)  # chunks per timed pass (each chunk writes to its own region)
    o0 = torch.empty(k * per * b0, dtype=torch.uint8, device="cuda")
    o1 = torch.empty(k * per * b1, dtype=torch.uint8, device="cuda") if b1 else None
    cnt = torch.zeros(k, dtype=torch.int64, device="cuda")
    masks = wl.masks()
    index = {c: i for i, c in enumerate(wl.coords)}
    offs = [(-1, 0, 0), (1, 0, 0), (0, 0, -1), (0, 0, 1), (0, -1, 0), (0, 1, 0)]
    o0p, o1p = o0.data_ptr(), (o1.data_ptr() if o1 is not None else 0)
    occp = occ.data_ptr()
    cp = d_coords.data_ptr()

    def one_pass():
        for i in range(k):
            # Chunk::new for the chunk and its loaded neighbours' occupancy is produced by
            # the same per-chunk generate launch (one chunk per launch)
            ctx.generate(cp + 12 * i, 1, occp + 4 * words * i, chunk_index_base=wl.index_base + i)
        for i in range(k):
            c = wl.coords[i]
            nb = []
            for d, (dx, dy, dz) in enumerate(offs):
                j = index.get((c[0] + dx, c[1] + dy, c[2] + dz))
                ok = (masks[i] >> d) & 1 and j is not None and j < k
                nb.append(occp + 4 * words * j if ok else None)
            ctx.mesh(occp + 4 * words * i, nb, c, o0p + i * per * b0,
                     (o1p + i * per * b1) if b1 else None, per, cnt.data_ptr() + 8 * i)

    with torch.cuda.stream(stream):
        one_pass()
        ctx.sync()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.plain_steps):
            one_pass()
        t1.record(stream)
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.plain_steps
    return {"value": k / (ms / 1e3), "unit": "chunks/s", "chunks_per_pass": k,
            "launches_per_chunk": 2, "ms_per_pass": ms}


def noise_kernel(ctx, wl, cfg, d_coords, n, stream, flush, args, torch):
    """The generation kernel alone (Chunk::new, src/chunk.rs:21-46): vox_generate writes the
    occupancy of every chunk (no halo) to a device pool; its noise FP32 work is samples x
    octaves x the formula's operation count, against the nominal FP32 instruction rate."""
    g = cfg.gen
    if g.kind not in (0, 1):
        return None
    N = cfg.chunk_size
    samples, dim = (N * N, 2) if g.kind == 0 else (N ** 3, 3)
    pool = torch.empty(n * ctx.sizes.occ_words_per_chunk, dtype=torch.int32, device="cuda")
    steps = max(3, args.steps // 4)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for _ in range(3):
            ctx.generate(d_coords, n, pool, chunk_index_base=wl.index_base)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            ctx.generate(d_coords, n, pool, chunk_index_base=wl.index_base)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    assert ctx.sync(raise_on_error=False) == 0
    ms = statistics.median(a.elapsed_time(b) for a, b in ev)
    ops = n * samples * g.octaves * NOISE_OPS[dim]
    achieved = ops / (ms / 1e3)
    return {"kernel": "k_generate", "ms": ms, "steps": steps, "chunks": n,
            "samples_per_chunk": samples, "octaves": g.octaves,
            "ops_per_sample_octave": NOISE_OPS[dim], "achieved_tops": achieved / 1e12,
            "peak_tops": FP32_OPS_NOMINAL / 1e12,
            "peak_source": "nominal FP32 instruction rate (FMA contraction off)",
            "frac": achieved / FP32_OPS_NOMINAL,
            "occupancy_bytes": n * ctx.sizes.occ_words_per_chunk * 4,
            "api": "vox_generate (occupancy to a device pool, L2 flushed before each step)"}


def mesh_from_occupancy(ctx, wl, cfg, d_coords, n, o0, o1, cap, total_faces, stream, flush, args,
                        torch, np):
    """The rebuild path (ChunkGenerator::process_rebuild_queue, src/chunk_builder.rs:89-112):
    vox_mesh_batch over occupancy already resident in a device pool (filled once by
    vox_generate, untimed), with the lateral neighbours' slots as the halo source."""
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
    steps = max(3, args.steps // 4)
    torch.cuda.synchronize()  # the buffers above were filled on the default stream
    with torch.cuda.stream(stream):
        ctx.generate(d_coords, n, pool, chunk_index_base=wl.index_base)
        for _ in range(3):
            ctx.mesh_batch(pool, n, d_slots, d_nbr, d_coords, n, o0, o1, cap, offs)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            ctx.mesh_batch(pool, n, d_slots, d_nbr, d_coords, n, o0, o1, cap, offs)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    assert ctx.sync(raise_on_error=False) == 0
    assert int(offs[-1].item()) == total_faces, "the rebuild path must emit the same faces"
    ms = statistics.median(a.elapsed_time(b) for a, b in ev)
    return {"value": n / (ms / 1e3), "unit": "chunks/s", "ms_per_step": ms, "steps": steps,
            "api": "vox_mesh_batch from device-resident occupancy (L2 flushed before each step)"}


def e2e_host(ctx, wl, masks, n, total_faces, b0, b1, args, np):
    """vox_gen_mesh_host with pinned host buffers: the coordinates and neighbour masks
    come from host memory and every emitted face and offset lands in host memory, all
    inside the timed call (the kernel reads and writes the page-locked buffers in place)."""
    import ctypes

    import voxgpu
    L = voxgpu.lib()

    def pinned(nbytes):
        p = ctypes.c_void_p()
        assert L.vox_host_alloc(max(16, nbytes), ctypes.byref(p)) == 0
        return p.value

    h_coords = pinned(n * 12)
    h_mask = pinned(n)
    ctypes.memmove(h_coords, np.asarray(wl.coords, np.int32).tobytes(), n * 12)
    ctypes.memmove(h_mask, np.asarray(masks, np.uint8).tobytes(), n)
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
    moved = n * 13 + (n + 1) * 8 + total_faces * (b0 + b1)
    return {"value": n / (ms / 1e3), "unit": "chunks/s", "ms_per_step": ms,
            "host_link_gbs": moved / (ms / 1e3) / 1e9,
            "h2d_bytes_per_step": n * 13, "d2h_bytes_per_step": (n + 1) * 8 + total_faces * (b0 + b1),
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
    for k in range(frames):
        ts = k / 60.0
        if paced:
            while voxgpu.Server.now() - t0 < ts:
                time.sleep(0.0005)
        eye, d = voxgpu.serving_camera(ts)
        srv.frame(voxgpu.camera_matrix(eye, d, zfar=zfar), eye)
    srv.drain()
    wall = voxgpu.Server.now() - t0
    st = srv.stats()
    srv.close()
    return {
        "frames": frames, "paced_60fps": paced, "requested": st.requested,
        "completed": st.completed, "launches": st.launches, "evicted": st.evicted,
        "p50_ms": st.latency_p50_ms, "p99_ms": st.latency_p99_ms, "max_ms": st.latency_max_ms,
        "chunks_per_s_busy": st.completed / st.busy_s if st.busy_s > 0 else None,
        "wall_s": wall, "frame_budget_ms": 1000.0 / 60,
    }


def run_serving(args):
    rank, world, local = dist_info()
    import torch
    torch.cuda.set_device(local)
    frames = args.frames
    res = serving_run(frames, args.paced)
    line = {
        "metric": METRIC, "value": res["chunks_per_s_busy"], "unit": "chunks/s",
        "n_gpus": 1, "steps": frames, "warmup": 0, "ms_per_step": res["wall_s"] * 1e3 / frames,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32",
        "data": "synthetic",
        "config": {"workload": "serving: simulated camera 20 u/s + 90 deg/s yaw, 60 frames/s, "
                               "heightmap-fbm 16^3 chunks, view radius 24, 24 GB LRU cache",
                   "paced": args.paced},
        "latency": res,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
