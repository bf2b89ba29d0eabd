"""Parity at the benchmark's own workload sizes and launch shapes (bit-exact).

The 3-D density workload (4096 chunks of 32^3, 638 MB of output) and the Bernoulli stress
workload (2048 chunks of 64^3, 98 GB of output) run exactly as bench.py runs them: the
whole batch resident on the device, the autotuned launch shape and output slab, replayed
from one captured graph (voxgpu.batch.BatchRun). Every chunk's face count is compared with
the oracle, and every chunk's vertex and index bytes through a per-chunk 64-bit digest
(oracle.chunk_digests of the GPU bytes against oracle.gen_mesh_digests, which restates
src/chunk.rs:21-245 and src/quad.rs:14-89 chunk by chunk on all host threads). Forced
shapes with several slabs of uneven size and both spill schedules cover what the
autotuner may not pick on a given box.
"""
import numpy as np
import pytest

from gpu_util import ctx_for, torch_cuda

pytestmark = pytest.mark.gpu


def verify_all_chunks(run, oracle, want_counts, want_dig, group):
    """Face counts of every chunk, then the digests of every chunk's bytes, `group` chunks
    at a time through one page-locked host buffer."""
    torch = torch_cuda()
    offs = run.host_offsets()
    assert int(offs[0]) == 0
    assert np.array_equal(np.diff(offs.astype(np.int64)), want_counts.astype(np.int64))
    n, b0, b1 = run.n, run.b0, run.b1
    starts = list(range(0, n, group))
    most = max(int(offs[min(n, a + group)] - offs[a]) for a in starts)
    h0 = torch.empty(max(most * b0, 16), dtype=torch.uint8, pin_memory=True)
    h1 = torch.empty(max(most * b1, 16), dtype=torch.uint8, pin_memory=True)
    for a in starts:
        b = min(n, a + group)
        lo, hi = int(offs[a]), int(offs[b])
        if hi > lo:
            h0[:(hi - lo) * b0].copy_(run.out0[lo * b0:hi * b0])
            if b1:
                h1[:(hi - lo) * b1].copy_(run.out1[lo * b1:hi * b1])
        torch.cuda.synchronize()
        got = oracle.chunk_digests(h0.numpy(), h1.numpy(), offs[a:b + 1] - offs[a], b0, b1)
        bad = np.nonzero(np.any(got != want_dig[a:b], axis=1))[0]
        assert bad.size == 0, f"chunks differing from the oracle: {(bad + a)[:8].tolist()}"


def refill_garbage(run):
    torch = torch_cuda()
    run.out0.fill_(0xAB)
    if run.out1 is not None:
        run.out1.fill_(0xCD)
    run.offsets.fill_(-1)
    torch.cuda.synchronize()


def test_density_workload_full_at_bench_shape(vox, oracle):
    """4096 chunks of 32^3, 3-D fBm density: the autotuned shape and slab, graph replays,
    then forced slabs of 1000 chunks (an uneven last slab) under the overlap and the phased
    schedules."""
    from voxgpu.batch import BatchRun
    wl = vox.workload("density")
    cfg = wl.config()
    coords, masks = list(wl.coords), wl.masks()
    want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, masks, wl.index_base)
    assert int(want_counts.sum()) > 5_000_000
    ctx = ctx_for(vox, cfg)
    run = BatchRun(ctx, coords, masks, wl.index_base, autotune=True, tune_iters=2)
    assert run.total_faces == int(want_counts.sum())
    refill_garbage(run)
    for _ in range(2):
        run.launch()
    ctx.sync()
    verify_all_chunks(run, oracle, want_counts, want_dig, group=len(coords))
    t = ctx.tuning()
    for sched in (vox.SCHEDULE_OVERLAP, vox.SCHEDULE_PHASED):
        ctx.set_tuning(t.threads, t.stage_faces, 0, sched, 1000)
        refill_garbage(run)
        ctx.gen_mesh_batch(run.d_coords, run.d_mask, run.n, run.out0, run.out1, run.cap,
                           run.offsets, chunk_index_base=wl.index_base)
        ctx.sync()
        verify_all_chunks(run, oracle, want_counts, want_dig, group=len(coords))
    run.close()
    ctx.close()


def test_stress_workload_full_at_bench_shape(vox, oracle):
    """2048 isolated chunks of 64^3, Bernoulli(0.5) from splitmix64(99 ^ index), the whole
    98 GB output resident: the autotuned shape and slab replayed from a graph, then forced
    1024-chunk slabs (overlap schedule, emission segments per chunk) and 768-chunk slabs
    (phased schedule, an uneven last slab). All 2048 chunks compared byte for byte."""
    from voxgpu.batch import BatchRun
    torch = torch_cuda()
    wl = vox.workload("stress")
    cfg = wl.config()
    coords = list(wl.coords)
    want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, None, wl.index_base)
    ctx = ctx_for(vox, cfg)
    run = BatchRun(ctx, coords, None, wl.index_base, autotune=True, tune_iters=1)
    assert run.total_faces == int(want_counts.sum())
    refill_garbage(run)
    run.launch()
    ctx.sync()
    verify_all_chunks(run, oracle, want_counts, want_dig, group=64)
    t = ctx.tuning()
    for sched, slab in ((vox.SCHEDULE_OVERLAP, 1024), (vox.SCHEDULE_PHASED, 768)):
        ctx.set_tuning(t.threads, t.stage_faces, 0, sched, slab)
        refill_garbage(run)
        ctx.gen_mesh_batch(run.d_coords, None, run.n, run.out0, run.out1, run.cap, run.offsets,
                           chunk_index_base=wl.index_base)
        ctx.sync()
        verify_all_chunks(run, oracle, want_counts, want_dig, group=64)
    run.close()
    ctx.close()
    torch.cuda.empty_cache()


def test_slabbed_batch_matches_one_launch_and_reports_capacity(vox, oracle):
    """A batch cut into slabs writes the same offsets and bytes as one launch, for every
    schedule and slab size (the heightmap batch, 1024 chunks of 16^3), and an output that
    ends inside a later slab is reported with the full offsets and the bytes before it."""
    from voxgpu.batch import BatchRun
    wl = vox.workload("heightmap")
    cfg = wl.config()
    coords, masks = list(wl.coords), wl.masks()
    want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, masks)
    ctx = ctx_for(vox, cfg)
    run = BatchRun(ctx, coords, masks, graph=False)
    t = ctx.tuning()
    for sched in (vox.SCHEDULE_LOOKBACK, vox.SCHEDULE_PHASED, vox.SCHEDULE_OVERLAP):
        for slab in (1, 100, 333, 512, 1023, 1024, 4096):
            ctx.set_tuning(t.threads, t.stage_faces, 0, sched, slab)
            refill_garbage(run)
            run.launch()
            ctx.sync()
            verify_all_chunks(run, oracle, want_counts, want_dig, group=len(coords))
    # capacity ends inside the last of three slabs, then inside the first
    offs_want = np.concatenate([[0], np.cumsum(want_counts)]).astype(np.uint64)
    for cap in (int(offs_want[900]) + 7, int(offs_want[100]) + 3):
        ctx.set_tuning(t.threads, t.stage_faces, 0, vox.SCHEDULE_OVERLAP, 400)
        refill_garbage(run)
        ctx.gen_mesh_batch(run.d_coords, run.d_mask, run.n, run.out0, run.out1, cap, run.offsets)
        assert ctx.sync(raise_on_error=False) == vox.VOX_ERR_CAPACITY
        assert np.array_equal(run.host_offsets(), offs_want)
        w0, w1, _ = oracle.gen_mesh_batch(cfg, coords, masks, cap=cap)
        torch = torch_cuda()
        torch.cuda.synchronize()
        assert np.array_equal(run.out0[:cap * 96].cpu().numpy(), w0)
        assert np.array_equal(run.out1[:cap * 24].cpu().numpy(), w1)
    run.close()
    ctx.close()


@pytest.mark.parametrize("name,limit", [("heightmap", 1024), ("density", 512), ("stress", 16)])
def test_rank_shards_match_the_oracle(vox, oracle, name, limit):
    """The weak-scaling shards bench.py gives each rank under torchrun (world size 2):
    every shard, meshed by the library with the bench's shape, equals the oracle on that
    shard's own coordinates and chunk indices (ranks run here one after the other; each
    needs no data from the other)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from voxgpu.batch import BatchRun
    seen = []
    for rank in (0, 1):
        wl = bench.shard_workload(vox.workload(name), rank, 2)
        cfg = wl.config()
        coords = list(wl.coords)[:limit]
        masks = None if wl.isolated else vox.neighbour_masks(coords)
        want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, masks, wl.index_base)
        ctx = ctx_for(vox, cfg)
        run = BatchRun(ctx, coords, masks, wl.index_base, autotune=False)
        refill_garbage(run)
        run.launch()
        ctx.sync()
        verify_all_chunks(run, oracle, want_counts, want_dig, group=min(len(coords), 256))
        seen.append((set(coords), wl.index_base))
        run.close()
        ctx.close()
    if name == "stress":
        assert seen[0][1] != seen[1][1]  # disjoint chunk-index ranges
    else:
        assert not (seen[0][0] & seen[1][0])  # disjoint chunk coordinates


@pytest.mark.parametrize("schedule", [0, 1, 2])
def test_slabbed_graph_replays(vox, oracle, schedule):
    """A captured graph holding several slab launches (300-chunk slabs of the 1024-chunk
    heightmap batch, the last one shorter) replays to the oracle's bytes, twice in a row."""
    from voxgpu.batch import BatchRun
    wl = vox.workload("heightmap")
    cfg = wl.config()
    coords, masks = list(wl.coords), wl.masks()
    want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, masks)
    ctx = ctx_for(vox, cfg)
    t = ctx.tuning()
    ctx.set_tuning(t.threads, t.stage_faces, 0, schedule, 300)
    run = BatchRun(ctx, coords, masks, graph=True)
    assert run.launches_per_step == 4
    for _ in range(2):
        refill_garbage(run)
        run.launch()
        ctx.sync()
        verify_all_chunks(run, oracle, want_counts, want_dig, group=len(coords))
    run.close()
    ctx.close()


@pytest.mark.parametrize("schedule", [0, 1, 2])
def test_slabbed_host_entry_point(vox, oracle, schedule):
    """vox_gen_mesh_host with 64-chunk slabs writes page-locked host buffers in place: the
    offsets and bytes of one launch, and a short output reports the full offsets."""
    from gpu_util import Pinned
    wl = vox.workload("heightmap")
    cfg = wl.config()
    n = 200
    coords = np.asarray(wl.coords[:n], np.int32)
    masks = np.asarray(vox.neighbour_masks(wl.coords[:n]), np.uint8)
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, wl.coords[:n], masks)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    t = ctx.tuning()
    ctx.set_tuning(t.threads, t.stage_faces, 0, schedule, 64)
    hc, hm = Pinned(vox, coords.nbytes), Pinned(vox, masks.nbytes)
    hc.view(np.int32)[:] = coords.reshape(-1)
    hm.view(np.uint8)[:] = masks
    h0, h1, ho = Pinned(vox, total * 96), Pinned(vox, total * 24), Pinned(vox, (n + 1) * 8)
    for _ in range(2):
        h0.a.fill(0xEE)
        ctx.gen_mesh_host(hc.ptr, hm.ptr, n, h0.ptr, h1.ptr, total, ho.ptr)
        assert np.array_equal(ho.view(np.uint64), woffs)
        assert np.array_equal(h0.view(np.uint8), w0) and np.array_equal(h1.view(np.uint8), w1)
    st = ctx.gen_mesh_host(hc.ptr, hm.ptr, n, h0.ptr, h1.ptr, total // 2, ho.ptr,
                           raise_on_error=False)
    assert st == vox.VOX_ERR_CAPACITY and np.array_equal(ho.view(np.uint64), woffs)
    assert np.array_equal(h0.view(np.uint8)[:(total // 2) * 96], w0[:(total // 2) * 96])
    for b in (hc, hm, h0, h1, ho):
        b.free()
    ctx.close()
