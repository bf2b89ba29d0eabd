"""The staged-halo path (vox_tuning.halo_staging = 1) against the oracle, bit for bit.

Every chunk of the batch is generated once into an occupancy pool, and for every loaded
neighbour outside it the one plane that the meshing reads; the neighbours are found by a
device hash lookup of the batch's coordinates, and the chunks are meshed from the pool with
each halo plane read from the neighbour's occupancy. The bytes must be those of the fused
launch, which regenerates the halos, and of the oracle, which generates every neighbour
from its coordinate.
"""
import numpy as np
import pytest

from gpu_util import Pinned, ctx_for, torch_cuda
from test_gpu_workloads_full import refill_garbage, verify_all_chunks

pytestmark = pytest.mark.gpu


def pool_tuning(ctx, schedule, slab=0):
    t = ctx.tuning()
    ctx.set_tuning(t.threads, t.stage_faces, 0, schedule, slab, 1)


@pytest.mark.parametrize("schedule", [0, 1, 2])
@pytest.mark.parametrize("graph", [False, True])
def test_pool_heightmap_batch(vox, oracle, schedule, graph):
    from voxgpu.batch import BatchRun
    wl = vox.workload("heightmap")
    cfg = wl.config()
    coords, masks = list(wl.coords), wl.masks()
    want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, masks)
    ctx = ctx_for(vox, cfg)
    for slab in (0, 300):
        pool_tuning(ctx, schedule, slab)
        run = BatchRun(ctx, coords, masks, graph=graph)
        assert run.tuning["halo"] == "pool"
        for _ in range(2):
            refill_garbage(run)
            run.launch()
            ctx.sync()
            verify_all_chunks(run, oracle, want_counts, want_dig, group=len(coords))
        run.close()
    ctx.close()


@pytest.mark.parametrize("cull", [0, 1])
def test_pool_density_with_neighbours_outside_the_batch(vox, oracle, cull):
    """A 4 x 3 x 4 block whose every chunk claims all its neighbours loaded: the chunks on
    the block's faces have neighbours outside the batch, generated into extra pool slots."""
    from voxgpu.batch import BatchRun
    wl = vox.workload("density")
    cfg = wl.config(cull_mode=cull)
    coords = vox.grid_coords(range(4, 8), range(7, 10), range(4, 8))
    masks = [0x3F if cull else 0x0F] * len(coords)
    want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, masks)
    ctx = ctx_for(vox, cfg)
    pool_tuning(ctx, 2)
    run = BatchRun(ctx, coords, masks, graph=False)
    refill_garbage(run)
    run.launch()
    ctx.sync()
    verify_all_chunks(run, oracle, want_counts, want_dig, group=len(coords))
    run.close()
    ctx.close()


@pytest.mark.parametrize("name,size", [("heightmap", 16), ("heightmap", 32), ("heightmap", 64),
                                       ("density", 8), ("density", 16), ("density", 64)])
@pytest.mark.parametrize("cull", [0, 1])
def test_pool_halo_planes_outside_the_batch(vox, oracle, name, size, cull):
    """Both noise generators at several chunk sizes, every neighbour claimed loaded: each
    chunk on the block's faces reads its halo from a plane generated alone into an extra
    pool slot (x, z and, with full culling, y planes on either side)."""
    from voxgpu.batch import BatchRun
    wl = vox.workload(name)
    cfg = vox.Workload(name, dict(wl.cfg_kwargs, chunk_size=size), ()).config(cull_mode=cull)
    # a block straddling the heightmap's surface (chunk y -1..1) or the density field's
    # (voxel y 224..319)
    if name == "heightmap":
        coords = vox.grid_coords(range(-2, 1), range(-1, 2), range(3, 5))
    else:
        ys = range(224 // size, max(320 // size, 224 // size + 2))
        coords = vox.grid_coords(range(128 // size, 128 // size + 3), ys,
                                 range(160 // size, 160 // size + 2))
    masks = [0x3F if cull else 0x0F] * len(coords)
    want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, masks)
    assert sum(want_counts) > 0
    ctx = ctx_for(vox, cfg)
    pool_tuning(ctx, 2)
    run = BatchRun(ctx, coords, masks, graph=False)
    assert run.tuning["halo"] == "pool"
    for _ in range(2):
        refill_garbage(run)
        run.launch()
        ctx.sync()
        verify_all_chunks(run, oracle, want_counts, want_dig, group=len(coords))
    run.close()
    ctx.close()


def test_pool_bernoulli_and_plain(vox, oracle):
    from voxgpu.batch import BatchRun
    for name, k, base in (("stress", 6, 1000), ("plain", 64, 0)):
        wl = vox.workload(name)
        cfg = wl.config()
        coords = list(wl.coords[:k])
        masks = None if wl.isolated else vox.neighbour_masks(coords)
        want_counts, want_dig = oracle.gen_mesh_digests(cfg, coords, masks, base)
        ctx = ctx_for(vox, cfg)
        pool_tuning(ctx, 2)
        run = BatchRun(ctx, coords, masks, base, graph=True)
        refill_garbage(run)
        run.launch()
        ctx.sync()
        verify_all_chunks(run, oracle, want_counts, want_dig, group=k)
        run.close()
        ctx.close()


def test_pool_host_entry_point(vox, oracle):
    """A context tuned to staged halos, through vox_gen_mesh_host: page-locked outputs keep
    the fused launch, pageable ones go through device buffers and the staged path."""
    wl = vox.workload("heightmap")
    cfg = wl.config()
    n = 200
    coords = np.asarray(wl.coords[:n], np.int32)
    masks = np.asarray(vox.neighbour_masks(wl.coords[:n]), np.uint8)
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, wl.coords[:n], masks)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    pool_tuning(ctx, 2, 64)
    hc, hm = Pinned(vox, coords.nbytes), Pinned(vox, masks.nbytes)
    hc.view(np.int32)[:] = coords.reshape(-1)
    hm.view(np.uint8)[:] = masks
    h0, h1, ho = Pinned(vox, total * 96), Pinned(vox, total * 24), Pinned(vox, (n + 1) * 8)
    ctx.gen_mesh_host(hc.ptr, hm.ptr, n, h0.ptr, h1.ptr, total, ho.ptr)
    assert np.array_equal(ho.view(np.uint64), woffs)
    assert np.array_equal(h0.view(np.uint8), w0) and np.array_equal(h1.view(np.uint8), w1)
    # pageable buffers take the device-buffer path
    p0, p1, po = np.zeros(total * 96, np.uint8), np.zeros(total * 24, np.uint8), np.zeros(n + 1, np.uint64)
    ctx.gen_mesh_host(coords, masks, n, p0, p1, total, po)
    assert np.array_equal(po, woffs) and np.array_equal(p0, w0) and np.array_equal(p1, w1)
    for b in (hc, hm, h0, h1, ho):
        b.free()
    ctx.close()


def test_pool_rejects_coordinates_beyond_the_key_range(vox):
    torch = torch_cuda()
    cfg = vox.workload("heightmap").config()
    ctx = ctx_for(vox, cfg)
    pool_tuning(ctx, 2)
    d_coords = torch.tensor([[0, 0, 0], [1 << 21, 0, 0]], dtype=torch.int32, device="cuda")
    offs = torch.zeros(3, dtype=torch.int64, device="cuda")
    ctx.gen_mesh_batch(d_coords, None, 2, None, None, 0, offs)
    assert ctx.sync(raise_on_error=False) == vox.VOX_ERR_INVALID
    ctx.set_tuning(ctx.tuning().threads, ctx.tuning().stage_faces, 0, 2, 0, 0)  # the fused path takes them
    ctx.gen_mesh_batch(d_coords, None, 2, None, None, 0, offs)
    assert ctx.sync(raise_on_error=False) == vox.VOX_ERR_CAPACITY  # no output room, offsets complete
    ctx.close()


def test_autotune_reports_a_halo_staging(vox):
    from voxgpu.batch import BatchRun
    wl = vox.workload("density")
    cfg = wl.config()
    coords = vox.grid_coords(range(4, 12), range(7, 10), range(4, 12))
    ctx = ctx_for(vox, cfg)
    run = BatchRun(ctx, coords, vox.neighbour_masks(coords), autotune=True, tune_iters=1,
                   graph=False)
    assert run.tuning["halo"] in ("pool", "regenerated")
    run.close()
    ctx.close()
