"""Parity of the CUDA path with the CPU oracle, through the C ABI (bit-exact).

Occupancy, face counts, offsets and every byte of the emitted vertex / index /
instance records must equal the oracle's on the same inputs (signed zeros included).
"""
import ctypes

import numpy as np
import pytest

from gpu_util import (Pinned, ctx_for, dev_bytes, gpu_gen_mesh, gpu_generate, to_dev, to_np,
                      use_schedule)

pytestmark = pytest.mark.gpu

LAYOUTS = [0, 1]  # vertex, instanced
SCHEDULES = [0, 1, 2]  # look-back, phased (cooperative launch), overlap


def small_coords():
    return [(0, 0, 0), (-1, 0, 0), (2, -1, 3), (-3, 1, -2), (5, 0, -7), (0, 2, 1)]


def gen_cfg(vox, kind, n, layout=0, cull=0):
    if kind == "height":
        return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_HEIGHTMAP,
                               octaves=4, seed=7, frequency=1 / 128, amplitude=48.0,
                               base_height=float(n // 2))
    if kind == "height1":
        return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_HEIGHTMAP,
                               octaves=1, seed=42, frequency=1 / 64, amplitude=12.0,
                               base_height=4.0)
    if kind == "density":
        return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_DENSITY,
                               octaves=3, seed=1234, frequency=1 / 96, y_ref=float(n // 2),
                               y_scale=1 / 64)
    if kind == "density4":  # the most octaves the lattice-table path takes
        return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_DENSITY,
                               octaves=4, seed=4321, frequency=1 / 64, y_ref=float(n // 2),
                               y_scale=1 / 48)
    if kind == "density1x":  # one octave, lattice cells 5 voxels wide (corner records reloaded
        # several times per block of x samples on the 32^3 path)
        return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_DENSITY,
                               octaves=1, seed=9, frequency=0.2, y_ref=float(n // 2),
                               y_scale=1 / 24)
    if kind == "density6":  # more octaves than the lattice-table path takes (per-sample path)
        return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_DENSITY,
                               octaves=6, seed=77, frequency=1 / 40, y_ref=float(n // 2),
                               y_scale=1 / 32)
    if kind == "densityhf":  # too many lattice corners for the tables (per-sample path)
        return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_DENSITY,
                               octaves=2, seed=5, frequency=0.7, y_ref=float(n // 2),
                               y_scale=1 / 16)
    if kind == "refdensity":  # the reference's parameters and fill rule (noise < 0 -> solid)
        return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_DENSITY,
                               octaves=3, seed=1, frequency=0.09, lacunarity=0.5, gain=2.5,
                               solid_below_zero=1)
    return vox.make_config(chunk_size=n, layout=layout, cull_mode=cull, kind=vox.GEN_BERNOULLI,
                           seed=99)


@pytest.mark.parametrize("n", [8, 16, 32, 64])
@pytest.mark.parametrize("kind", ["height", "height1", "density", "density4", "density1x",
                                  "density6", "densityhf", "refdensity", "bernoulli"])
def test_generate_matches_oracle(vox, oracle, n, kind):
    cfg = gen_cfg(vox, kind, n)
    coords = small_coords()
    got = gpu_generate(vox, cfg, coords, index_base=11)
    for i, c in enumerate(coords):
        want = oracle.cubes_to_occ(n, oracle.generate_cubes(cfg, c, 11 + i))
        assert np.array_equal(got[i], want), (kind, n, c)


@pytest.mark.parametrize("n", [8, 16, 32, 64])
def test_cubes_occ_roundtrip(vox, oracle, n):
    rng = np.random.default_rng(n)
    cfg = vox.make_config(chunk_size=n)
    k = 3
    cubes = rng.choice(np.array([0, 1, 2], np.uint8), size=k * n ** 3, p=[0.4, 0.1, 0.5])
    ctx = ctx_for(vox, cfg)
    words = ctx.sizes.occ_words_per_chunk
    d_c = to_dev(cubes)
    d_o = dev_bytes(k * words * 4)
    ctx.cubes_to_occ(d_c, k, d_o)
    occ = to_np(d_o, k * words * 4).view(np.uint32).reshape(k, words)
    for i in range(k):
        assert np.array_equal(occ[i], oracle.cubes_to_occ(n, cubes[i * n ** 3:(i + 1) * n ** 3]))
    d_back = dev_bytes(k * n ** 3)
    ctx.occ_to_cubes(d_o, k, d_back)
    back = to_np(d_back, k * n ** 3)
    assert np.array_equal(back, np.where(cubes == 2, 2, 0).astype(np.uint8))


def patterns(n, rng):
    """Occupancy patterns of the known-answer tests plus random densities."""
    idx = np.arange(n ** 3)
    x, z, y = idx % n, (idx // n) % n, idx // (n * n)
    out = {
        "air": np.full(n ** 3, 2, np.uint8),
        "solid": np.zeros(n ** 3, np.uint8),
        "checker": np.where((x + y + z) % 2 == 0, 0, 2).astype(np.uint8),
        "one": np.where((x == 3) & (y == 2) & (z == n - 1), 0, 2).astype(np.uint8),
    }
    for p in (0.1, 0.5, 0.9):
        out[f"rand{p}"] = np.where(rng.random(n ** 3) < p, 0, 2).astype(np.uint8)
    return out


def run_mesh_single(vox, cfg, cubes, adj, coord):
    n = cfg.chunk_size
    ctx = ctx_for(vox, cfg)
    occ = oracle_occ = None
    import vox_oracle
    oracle_occ = vox_oracle.cubes_to_occ(n, cubes)
    occ = to_dev(oracle_occ)
    nb = [None if a is None else to_dev(vox_oracle.cubes_to_occ(n, a)) for a in adj]
    cap = ctx.sizes.max_faces_per_chunk
    b0, b1 = ctx.sizes.bytes_per_face_out0, ctx.sizes.bytes_per_face_out1
    o0 = dev_bytes(cap * b0, 0xEE)
    o1 = dev_bytes(cap * b1, 0xEE)
    cnt = to_dev(np.zeros(1, np.uint64))
    ctx.mesh(occ, nb, coord, o0, o1 if b1 else None, cap, cnt)
    ctx.sync()
    c = int(to_np(cnt)[0])
    r = to_np(o0, c * b0), (to_np(o1, c * b1) if b1 else np.zeros(0, np.uint8)), c
    ctx.close()
    return r


@pytest.mark.parametrize("n", [8, 16, 32, 64])
@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("cull", [0, 1])
def test_mesh_single_matches_oracle(vox, oracle, n, layout, cull):
    rng = np.random.default_rng(100 * n + 10 * layout + cull)
    cfg = vox.make_config(chunk_size=n, layout=layout, cull_mode=cull)
    pats = patterns(n, rng)
    names = list(pats)
    for k, name in enumerate(names):
        cubes = pats[name]
        adj = []
        for d in range(6):
            choice = rng.integers(0, 3)
            adj.append(None if choice == 0 else pats[names[rng.integers(0, len(names))]])
        coord = (int(rng.integers(-50, 50)), int(rng.integers(-5, 5)), int(rng.integers(-50, 50)))
        w0, w1, wc = oracle.mesh_chunk(cfg, coord, cubes, adj)
        g0, g1, gc = run_mesh_single(vox, cfg, cubes, adj, coord)
        assert gc == wc, (name, gc, wc)
        assert np.array_equal(g0, w0), name
        assert np.array_equal(g1, w1), name


@pytest.mark.parametrize("n", [16, 32])
@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_mesh_batch_pool_matches_oracle(vox, oracle, n, layout, schedule):
    rng = np.random.default_rng(7 + n + layout)
    cfg = vox.make_config(chunk_size=n, layout=layout)
    slots = 9
    pool_cubes = [np.where(rng.random(n ** 3) < p, 0, 2).astype(np.uint8)
                  for p in rng.uniform(0.05, 0.95, slots)]
    pool = np.concatenate([oracle.cubes_to_occ(n, c) for c in pool_cubes])
    m = 14
    sl = rng.integers(0, slots, m).astype(np.int32)
    nbr = rng.integers(-1, slots, (m, 6)).astype(np.int32)
    coords = [(int(a), 0, int(b)) for a, b in rng.integers(-20, 20, (m, 2))]
    ctx = ctx_for(vox, cfg)
    use_schedule(ctx, schedule)
    b0, b1 = ctx.sizes.bytes_per_face_out0, ctx.sizes.bytes_per_face_out1
    cap = ctx.sizes.max_faces_per_chunk * m
    o0, o1 = dev_bytes(cap * b0), dev_bytes(cap * b1)
    offs = to_dev(np.zeros(m + 1, np.uint64))
    ctx.mesh_batch(to_dev(pool), slots, to_dev(sl), to_dev(nbr), to_dev(np.array(coords, np.int32)),
                   m, o0, o1 if b1 else None, cap, offs)
    ctx.sync()
    offsets = to_np(offs)
    total = int(offsets[m])
    g0 = to_np(o0, total * b0)
    g1 = to_np(o1, total * b1) if b1 else None
    acc = 0
    for i in range(m):
        adj = [None if nbr[i, d] < 0 else pool_cubes[nbr[i, d]] for d in range(6)]
        w0, w1, wc = oracle.mesh_chunk(cfg, coords[i], pool_cubes[sl[i]], adj)
        assert int(offsets[i]) == acc
        assert np.array_equal(g0[acc * b0:(acc + wc) * b0], w0)
        if b1:
            assert np.array_equal(g1[acc * b1:(acc + wc) * b1], w1)
        acc += wc
    assert acc == total
    ctx.close()


def compare_batch(vox, oracle, cfg, coords, masks, index_base=0, schedule=None):
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks, index_base)
    total = int(woffs[-1])
    g0, g1, goffs, _ = gpu_gen_mesh(vox, cfg, coords, masks, index_base, cap=max(total, 1),
                                    schedule=schedule)
    assert np.array_equal(goffs, woffs)
    assert np.array_equal(g0, w0)
    assert np.array_equal(g1, w1)
    return total


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_plain_workload_full(vox, oracle, layout, schedule):
    """8x8 chunks of 32^3 around the origin, 2-D Perlin heightmap (the CPU-runnable case)."""
    wl = vox.workload("plain")
    total = compare_batch(vox, oracle, wl.config(layout=layout), wl.coords, wl.masks(),
                          schedule=schedule)
    assert total > 0


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_heightmap_workload_full(vox, oracle, layout, schedule):
    """32x32 chunks of 16^3, 2-D fBm: all-air, all-solid and surface chunks."""
    wl = vox.workload("heightmap")
    total = compare_batch(vox, oracle, wl.config(layout=layout), wl.coords, wl.masks(),
                          schedule=schedule)
    assert total > 0


@pytest.mark.parametrize("cull", [0, 1])
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_density_workload_slab(vox, oracle, cull, schedule):
    """A 4x3x4 block of the 3-D density terrain around its surface (y = 256)."""
    wl = vox.workload("density")
    coords = vox.grid_coords(range(4, 8), range(7, 10), range(4, 8))
    total = compare_batch(vox, oracle, wl.config(cull_mode=cull), coords,
                          vox.neighbour_masks(coords, full6=bool(cull)), schedule=schedule)
    assert total > 0


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_stress_workload_sample(vox, oracle, layout, schedule):
    """Four isolated 64^3 Bernoulli(0.5) chunks (index base 1000)."""
    wl = vox.workload("stress")
    coords = [(i, 0, 0) for i in range(4)]
    total = compare_batch(vox, oracle, wl.config(layout=layout), coords, None, index_base=1000,
                          schedule=schedule)
    assert total > 4 * 300_000


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_capacity_overflow_reports_and_keeps_prefix(vox, oracle, schedule):
    wl = vox.workload("heightmap")
    cfg = wl.config()
    coords = wl.coords[:64]
    masks = vox.neighbour_masks(coords)
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks)
    total = int(woffs[-1])
    cap = total // 3
    g0, g1, goffs, st = gpu_gen_mesh(vox, cfg, coords, masks, cap=cap, expect_status=True,
                                     schedule=schedule)
    assert st == vox.VOX_ERR_CAPACITY
    assert np.array_equal(goffs, woffs)
    assert np.array_equal(g0, w0[:cap * 96]) and np.array_equal(g1, w1[:cap * 24])


def test_chunk_bytes_independent_of_batch(vox, oracle):
    """A chunk's mesh is the same alone and inside any batch (indices are chunk-local)."""
    wl = vox.workload("plain")
    cfg = wl.config()
    coords = list(wl.coords)
    masks = wl.masks()
    a0, a1, aoffs, _ = gpu_gen_mesh(vox, cfg, coords, masks, cap=2_000_000)
    for k in (0, 17, 63):
        s0, s1, soffs, _ = gpu_gen_mesh(vox, cfg, [coords[k]], [masks[k]], cap=200_000)
        lo, hi = int(aoffs[k]), int(aoffs[k + 1])
        assert hi - lo == int(soffs[1])
        assert np.array_equal(a0[lo * 96:hi * 96], s0)
        assert np.array_equal(a1[lo * 24:hi * 24], s1)


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_repeat_launches_identical(vox, schedule):
    """Back-to-back launches on one context (epoch-tagged look-back, queue words reset by
    the last ticket) give the same bytes: 300 launches without a host sync in between,
    direct and as graph replays, as in a timed loop."""
    wl = vox.workload("heightmap")
    cfg = wl.config()
    ctx = ctx_for(vox, cfg)
    use_schedule(ctx, schedule)
    n = len(wl.coords)
    d_coords = to_dev(np.asarray(wl.coords, np.int32))
    d_mask = to_dev(np.asarray(wl.masks(), np.uint8))
    cap = 3_000_000
    o0, o1 = dev_bytes(cap * 96), dev_bytes(cap * 24)
    offs = to_dev(np.zeros(n + 1, np.uint64))
    g = ctx.capture_graph(d_coords, d_mask, n, o0, o1, cap, offs)
    digests = []
    for rep in range(6):
        for _ in range(50):
            if rep % 2:
                g.launch()
            else:
                ctx.gen_mesh_batch(d_coords, d_mask, n, o0, o1, cap, offs)
        assert ctx.sync(raise_on_error=False) == vox.VOX_OK, rep
        total = int(to_np(offs)[n])
        digests.append((total, hash(to_np(o0, total * 96).tobytes()),
                        hash(to_np(o1, total * 24).tobytes())))
    assert len(set(digests)) == 1
    g.close()
    ctx.close()


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("layout", LAYOUTS)
def test_host_entry_point_pinned_zero_copy(vox, oracle, schedule, layout):
    """Page-locked host buffers: the kernel writes faces and offsets in host memory."""
    wl = vox.workload("heightmap")
    cfg = wl.config(layout=layout)
    n = 200
    coords = np.asarray(wl.coords[:n], np.int32)
    masks = np.asarray(vox.neighbour_masks(wl.coords[:n]), np.uint8)
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, wl.coords[:n], masks)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    use_schedule(ctx, schedule)
    b0, b1 = ctx.sizes.bytes_per_face_out0, ctx.sizes.bytes_per_face_out1
    hc, hm = Pinned(vox, coords.nbytes), Pinned(vox, masks.nbytes)
    hc.view(np.int32)[:] = coords.reshape(-1)
    hm.view(np.uint8)[:] = masks
    h0, h1, ho = Pinned(vox, total * b0), Pinned(vox, max(total * b1, 16)), Pinned(vox, (n + 1) * 8)
    p1 = h1.ptr if b1 else None
    for rep in range(2):
        h0.a.fill(0xEE)
        ctx.gen_mesh_host(hc.ptr, hm.ptr, n, h0.ptr, p1, total, ho.ptr)
        assert np.array_equal(ho.view(np.uint64), woffs), rep
        assert np.array_equal(h0.view(np.uint8), w0), rep
        if b1:
            assert np.array_equal(h1.view(np.uint8), w1), rep
    # pageable inputs with page-locked outputs
    ctx.gen_mesh_host(coords, masks, n, h0.ptr, p1, total, ho.ptr)
    assert np.array_equal(h0.view(np.uint8), w0) and np.array_equal(ho.view(np.uint64), woffs)
    st = ctx.gen_mesh_host(hc.ptr, hm.ptr, n, h0.ptr, p1, total - 1, ho.ptr,
                           raise_on_error=False)
    assert st == vox.VOX_ERR_CAPACITY and int(ho.view(np.uint64)[-1]) == total
    assert np.array_equal(h0.view(np.uint8)[:(total - 1) * b0], w0[:(total - 1) * b0])
    for b in (hc, hm, h0, h1, ho):
        b.free()
    ctx.close()


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_graph_replay_with_inputs_rewritten_in_place(vox, oracle, schedule):
    """A captured batch replays exactly; rewriting the inputs between replays changes the
    result exactly as a fresh launch would, and other context calls in between do not
    disturb the graph."""
    wl = vox.workload("heightmap")
    cfg = wl.config()
    n = 256
    sets = [list(wl.coords[:n]), list(wl.coords[n:2 * n]), list(wl.coords[:n])]
    want = [oracle.gen_mesh_batch(cfg, c, vox.neighbour_masks(c)) for c in sets[:2]]
    cap = max(int(w[2][-1]) for w in want)
    ctx = ctx_for(vox, cfg)
    use_schedule(ctx, schedule)
    d_coords = to_dev(np.asarray(sets[0], np.int32))
    d_mask = to_dev(np.asarray(vox.neighbour_masks(sets[0]), np.uint8))
    o0, o1 = dev_bytes(cap * 96), dev_bytes(cap * 24)
    offs = to_dev(np.zeros(n + 1, np.uint64))
    g = ctx.capture_graph(d_coords, d_mask, n, o0, o1, cap, offs)
    for k, coords in enumerate(sets):
        d_coords.copy_(to_dev(np.asarray(coords, np.int32)))
        d_mask.copy_(to_dev(np.asarray(vox.neighbour_masks(coords), np.uint8)))
        for rep in range(2):
            o0.fill_(0)
            g.launch()
            ctx.sync()
            w0, w1, woffs = want[k % 2]
            total = int(woffs[-1])
            assert np.array_equal(to_np(offs), woffs), (k, rep)
            assert np.array_equal(to_np(o0, total * 96), w0), (k, rep)
            assert np.array_equal(to_np(o1, total * 24), w1), (k, rep)
        # an ordinary launch on the same context between replays; the larger batch grows
        # the context's own scratch (the graph keeps its own)
        big = vox.grid_coords(range(0, 40), [0], range(0, 40))
        ctx.gen_mesh_batch(to_dev(np.asarray(big, np.int32)), None, len(big), dev_bytes(16),
                           dev_bytes(16), 0, to_dev(np.zeros(len(big) + 1, np.uint64)))
        assert ctx.sync(raise_on_error=False) == vox.VOX_ERR_CAPACITY
    g.close()
    ctx.close()


@pytest.mark.parametrize("ctas", [0, 1])
def test_host_entry_point_interleaved_emission(vox, oracle, ctas):
    """Host outputs with more chunks than two waves of CTAs: the overlap kernel interleaves
    emission items with generation items (emission two waves behind), and the bytes are
    the oracle's. One CTA per SM makes the waves short, so most items interleave."""
    wl = vox.workload("heightmap")
    cfg = wl.config()
    coords = vox.grid_coords(range(-20, 20), [0], range(-20, 20))  # 1600 chunks of 16^3
    n = len(coords)
    masks = np.asarray(vox.neighbour_masks(coords), np.uint8)
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    t = ctx.tuning()
    ctx.set_tuning(t.threads, t.stage_faces, ctas, vox.SCHEDULE_OVERLAP)
    hc, hm = Pinned(vox, n * 12), Pinned(vox, n)
    hc.view(np.int32)[:] = np.asarray(coords, np.int32).reshape(-1)
    hm.view(np.uint8)[:] = masks
    h0, h1, ho = Pinned(vox, total * 96), Pinned(vox, total * 24), Pinned(vox, (n + 1) * 8)
    for rep in range(2):
        h0.a.fill(0xEE)
        ctx.gen_mesh_host(hc.ptr, hm.ptr, n, h0.ptr, h1.ptr, total, ho.ptr)
        assert np.array_equal(ho.view(np.uint64), woffs), rep
        assert np.array_equal(h0.view(np.uint8), w0), rep
        assert np.array_equal(h1.view(np.uint8), w1), rep
    for b in (hc, hm, h0, h1, ho):
        b.free()
    ctx.close()


@pytest.mark.parametrize("kind", ["height", "density"])
def test_small_chunks_every_launch_shape(vox, oracle, kind):
    """8^3 chunks (one- and two-warp CTAs) in every schedule, staging window and CTAs per
    SM, with fewer chunks than CTAs (emission split into segments) and with more."""
    cfg = gen_cfg(vox, kind, 8)
    tried = 0
    for m in (40, 3000):
        coords = vox.grid_coords(range(0, 5 if m == 40 else 60), range(0, 1 if m == 40 else 1),
                                 range(0, 8 if m == 40 else 50))[:m]
        masks = vox.neighbour_masks(coords)
        w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks)
        total = int(woffs[-1])
        ctx = ctx_for(vox, cfg)
        d_coords = to_dev(np.asarray(coords, np.int32))
        d_mask = to_dev(np.asarray(masks, np.uint8))
        o0, o1 = dev_bytes(max(total, 1) * 96), dev_bytes(max(total, 1) * 24)
        offs = to_dev(np.zeros(len(coords) + 1, np.uint64))
        for sched in SCHEDULES:
            for threads in threads_options(8):
                for stage in (0, 32, 64):
                    for cps in (0, 1):
                        ctx.set_tuning(threads, stage, cps, sched)
                        o0.fill_(0x5A)
                        ctx.gen_mesh_batch(d_coords, d_mask, len(coords), o0, o1, total, offs)
                        ctx.sync()
                        tag = (m, sched, threads, stage, cps)
                        assert np.array_equal(to_np(offs), woffs), tag
                        assert np.array_equal(to_np(o0, total * 96), w0), tag
                        assert np.array_equal(to_np(o1, total * 24), w1), tag
                        tried += 1
        ctx.close()
    assert tried == 2 * len(SCHEDULES) * 2 * 3 * 2


def test_host_entry_point_matches_oracle(vox, oracle):
    wl = vox.workload("plain")
    cfg = wl.config()
    coords = np.asarray(wl.coords, np.int32)
    masks = np.asarray(wl.masks(), np.uint8)
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, wl.coords, masks)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    h0 = np.zeros(total * 96, np.uint8)
    h1 = np.zeros(total * 24, np.uint8)
    hoffs = np.zeros(len(coords) + 1, np.uint64)
    ctx.gen_mesh_host(coords, masks, len(coords), h0, h1, total, hoffs)
    assert np.array_equal(hoffs, woffs)
    assert np.array_equal(h0, w0) and np.array_equal(h1, w1)
    # too small: the status says so and the offsets still give the required size
    st = ctx.gen_mesh_host(coords, masks, len(coords), h0, h1, total - 1, hoffs,
                           raise_on_error=False)
    assert st == vox.VOX_ERR_CAPACITY and int(hoffs[-1]) == total
    ctx.close()


def test_frustum_matches_oracle(vox, oracle):
    from test_oracle_kat import perspective_look
    rng = np.random.default_rng(3)
    cfg = vox.make_config(chunk_size=32)
    ctx = ctx_for(vox, cfg)
    coords = rng.integers(-12, 12, (5000, 3)).astype(np.int32)
    d_coords = to_dev(coords)
    vis = dev_bytes(len(coords))
    for t in range(8):
        eye = rng.uniform(-100, 100, 3)
        fwd = rng.standard_normal(3)
        M = perspective_look(eye, fwd, fovy=float(rng.uniform(0.5, 2.0)), far=float(rng.uniform(50, 400)))
        planes = vox.frustum_planes(M.T.reshape(16))
        assert np.array_equal(np.array(planes, np.float32), oracle.frustum_planes(M.T.reshape(16)))
        ctx.frustum_cull(planes, d_coords, len(coords), vis)
        got = to_np(vis, len(coords))
        want = np.array([oracle.frustum_contains(planes, tuple(c), 32) for c in coords], np.uint8)
        assert np.array_equal(got, want)
        assert 0 < want.sum() < len(coords) or t > 0
    ctx.close()


@pytest.mark.parametrize("layout", LAYOUTS)
def test_draw_list_matches_oracle(vox, oracle, layout):
    """World::render as an indirect draw list: the visible chunks with faces, in chunk
    order, with the vertex / instance ranges of their meshes."""
    wl = vox.workload("heightmap")
    cfg = wl.config(layout=layout)
    coords = list(wl.coords[:600])
    masks = vox.neighbour_masks(coords)
    _, _, offs = oracle.gen_mesh_batch(cfg, coords, masks)
    m = vox.camera_matrix((100.0, 40.0, 60.0), (-1.0, -0.3, -0.4), zfar=300.0)
    planes = oracle.frustum_planes(m)
    want = []
    for i, c in enumerate(coords):
        f0, nf = int(offs[i]), int(offs[i + 1]) - int(offs[i])
        if nf > 0 and oracle.frustum_contains(planes, c, 16):
            want.append((6, nf, 0, 0, f0) if layout == 1 else (6 * nf, 1, 6 * f0, 4 * f0, 0))
    assert 0 < len(want) < len(coords)
    ctx = ctx_for(vox, cfg)
    d_draws = to_dev(np.zeros((len(coords), 5), np.uint32))
    d_count = to_dev(np.zeros(1, np.uint32))
    ctx.draw_list(planes, to_dev(np.asarray(coords, np.int32)), to_dev(offs), len(coords),
                  d_draws, d_count)
    ctx.sync()
    k = int(to_np(d_count)[0])
    got = to_np(d_draws)[:k].astype(np.int64)
    assert k == len(want)
    assert np.array_equal(got, np.asarray(want, np.int64).reshape(-1, 5))
    ctx.close()


def test_invalid_arguments_rejected(vox):
    cfg = vox.make_config(chunk_size=16)
    ctx = ctx_for(vox, cfg)
    with pytest.raises(vox.VoxError) as e:
        ctx.gen_mesh_batch(None, None, 4, None, None, 0, None)
    assert e.value.status == vox.VOX_ERR_INVALID
    d_coords = to_dev(np.zeros((2, 3), np.int32))
    offs = to_dev(np.zeros(3, np.uint64))
    bad = dev_bytes(4096)
    with pytest.raises(vox.VoxError):  # misaligned vertex output
        ctx.gen_mesh_batch(d_coords, None, 2, bad.data_ptr() + 4, bad, 10, offs)
    ctx.close()


def threads_options(n):
    return {8: (32, 64), 16: (128, 256), 32: (256, 512), 64: (512, 1024)}[n]


@pytest.mark.parametrize("wlname,sub,layout", [("heightmap", 160, 0), ("heightmap", 160, 1),
                                               ("plain", 64, 0), ("stress", 2, 0),
                                               ("stress", 2, 1)])
def test_every_launch_shape_is_bit_exact(vox, oracle, wlname, sub, layout):
    """CTA size, staging window (or direct stores) and CTAs per SM change only the speed."""
    wl = vox.workload(wlname)
    cfg = wl.config(layout=layout)
    n = cfg.chunk_size
    coords = list(wl.coords[:sub])
    masks = None if wl.isolated else vox.neighbour_masks(coords)
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    b0, b1 = ctx.sizes.bytes_per_face_out0, ctx.sizes.bytes_per_face_out1
    d_coords = to_dev(np.asarray(coords, np.int32))
    d_mask = None if masks is None else to_dev(np.asarray(masks, np.uint8))
    o0, o1 = dev_bytes(total * b0), dev_bytes(max(total * b1, 16))
    offs = to_dev(np.zeros(len(coords) + 1, np.uint64))
    tried = 0
    for sched in (vox.SCHEDULE_LOOKBACK, vox.SCHEDULE_PHASED, vox.SCHEDULE_OVERLAP):
        for threads in threads_options(n):
            for stage in (0, 32, 64):
                for cps in (0, 2):
                    try:
                        ctx.set_tuning(threads, stage, cps, sched)
                    except vox.VoxError:
                        continue  # the staging window does not fit in shared memory
                    for rep in range(2):  # the second launch reuses the reset queues
                        o0.fill_(0x5A)
                        offs.fill_(0)
                        ctx.gen_mesh_batch(d_coords, d_mask, len(coords), o0, o1 if b1 else None,
                                           total, offs)
                        ctx.sync()
                        tag = (sched, threads, stage, cps, rep)
                        assert np.array_equal(to_np(offs), woffs), tag
                        assert np.array_equal(to_np(o0, total * b0), w0), tag
                        if b1:
                            assert np.array_equal(to_np(o1, total * b1), w1), tag
                    tried += 1
    assert tried >= 10
    ctx.close()


def test_autotune_picks_a_valid_shape(vox, oracle):
    wl = vox.workload("heightmap")
    cfg = wl.config()
    coords = list(wl.coords)
    masks = wl.masks()
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    d_coords = to_dev(np.asarray(coords, np.int32))
    d_mask = to_dev(np.asarray(masks, np.uint8))
    o0, o1 = dev_bytes(total * 96), dev_bytes(total * 24)
    offs = to_dev(np.zeros(len(coords) + 1, np.uint64))
    t = ctx.autotune(d_coords, d_mask, len(coords), o0, o1, total, offs, iters=2)
    assert t.threads in threads_options(16)
    assert t.stage_faces in (0, 32, 64)
    got = ctx.tuning()
    assert t.schedule in (vox.SCHEDULE_LOOKBACK, vox.SCHEDULE_PHASED, vox.SCHEDULE_OVERLAP)
    assert (got.threads, got.stage_faces, got.ctas_per_sm, got.schedule) == (
        t.threads, t.stage_faces, t.ctas_per_sm, t.schedule)
    o0.fill_(0)
    ctx.gen_mesh_batch(d_coords, d_mask, len(coords), o0, o1, total, offs)
    ctx.sync()
    assert np.array_equal(to_np(o0, total * 96), w0) and np.array_equal(to_np(o1, total * 24), w1)
    ctx.close()


def test_bounded_wait_times_out_and_context_survives(vox, oracle):
    """A look-back whose predecessor never publishes returns VOX_ERR_TIMEOUT (no hang, no
    trap); the next batch on the same context is still exact."""
    wl = vox.workload("plain")
    cfg = wl.config()
    ctx = ctx_for(vox, cfg)
    assert ctx.selftest_lookback_timeout(2000) == vox.VOX_ERR_TIMEOUT
    assert ctx.sync(raise_on_error=False) == vox.VOX_OK  # the error was reported once
    coords = list(wl.coords[:8])
    masks = vox.neighbour_masks(coords)
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks)
    total = int(woffs[-1])
    d_coords = to_dev(np.asarray(coords, np.int32))
    d_mask = to_dev(np.asarray(masks, np.uint8))
    o0, o1 = dev_bytes(total * 96), dev_bytes(total * 24)
    offs = to_dev(np.zeros(len(coords) + 1, np.uint64))
    ctx.gen_mesh_batch(d_coords, d_mask, len(coords), o0, o1, total, offs)
    ctx.sync()
    assert np.array_equal(to_np(o0, total * 96), w0)
    ctx.close()


@pytest.mark.parametrize("stage", [0, 32, 64])
def test_single_chunk_direct_and_staged(vox, oracle, stage):
    rng = np.random.default_rng(11)
    cfg = vox.make_config(chunk_size=32)
    cubes = np.where(rng.random(32 ** 3) < 0.5, 0, 2).astype(np.uint8)
    w0, w1, wc = oracle.mesh_chunk(cfg, (3, -2, 5), cubes, [None] * 6)
    ctx = ctx_for(vox, cfg)
    ctx.set_tuning(512, stage, 0)
    occ = to_dev(oracle.cubes_to_occ(32, cubes))
    o0, o1 = dev_bytes(wc * 96), dev_bytes(wc * 24)
    cnt = to_dev(np.zeros(1, np.uint64))
    ctx.mesh(occ, [None] * 6, (3, -2, 5), o0, o1, wc, cnt)
    ctx.sync()
    assert int(to_np(cnt)[0]) == wc
    assert np.array_equal(to_np(o0, wc * 96), w0) and np.array_equal(to_np(o1, wc * 24), w1)
    ctx.close()


@pytest.mark.parametrize("view", [0, 1])
def test_raster_matches_oracle(vox, oracle, view):
    """The headless rasteriser renders the plain workload's mesh byte for byte like the
    oracle's rasteriser (order-independent depth resolution)."""
    wl = vox.workload("plain")
    cfg = wl.config()
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, wl.coords, wl.masks())
    faces = int(woffs[-1])
    eye, d = [((60.0, 45.0, 70.0), (-0.6, -0.45, -0.65)), ((0.5, 20.0, 0.5), (0.3, -0.25, 1.0))][view]
    m = vox.camera_matrix(eye, d, zfar=400.0)  # Camera::update_global_matrix, column-major
    W, H = 320, 180
    want = oracle.raster(m, w0, w1, faces, W, H, cfg.texture_index)
    bg = (want.reshape(-1, 4) == np.array([26, 51, 77, 255], np.uint8)).all(1).mean()
    assert 0.2 < bg < 0.9 and len(np.unique(want.reshape(-1, 4), axis=0)) >= 5
    ctx = ctx_for(vox, cfg)
    d0, d1 = to_dev(np.frombuffer(w0, np.uint8)), to_dev(np.frombuffer(w1, np.uint8))
    keys = dev_bytes(W * H * 8)
    rgba = dev_bytes(W * H * 4)
    lib = vox.lib()
    mm = (ctypes.c_float * 16)(*[float(v) for v in np.asarray(m, np.float32).reshape(16)])
    st = lib.vox_raster(ctx._h, ctypes.addressof(mm), d0.data_ptr(), d1.data_ptr(), faces, W, H,
                        keys.data_ptr(), rgba.data_ptr())
    assert st == vox.VOX_OK
    ctx.sync()
    got = to_np(rgba, W * H * 4).reshape(H, W, 4)
    assert np.array_equal(got, want)
    ctx.close()


@pytest.mark.parametrize("case", range(24))
def test_randomized_batches_match_oracle(vox, oracle, case):
    """Seeded random configurations: chunk size, generator, layout, culling, coordinates,
    neighbour masks, schedule and launch shape all drawn per case."""
    rng = np.random.default_rng(1000 + case)
    n = int(rng.choice([8, 16, 32, 64]))
    kind = str(rng.choice(["height", "height1", "density", "refdensity", "bernoulli"]))
    layout = int(rng.integers(0, 2))
    cull = int(rng.integers(0, 2))
    cfg = gen_cfg(vox, kind, n, layout=layout, cull=cull)
    m = int(rng.integers(1, 9 if n == 64 else 25))
    coords = [tuple(int(v) for v in rng.integers(-6, 6, 3)) for _ in range(m)]
    masks = [int(v) for v in rng.integers(0, 64 if cull else 16, m)]
    base = int(rng.integers(0, 10_000))
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks, base)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    threads = threads_options(n)[int(rng.integers(0, 2))]
    stage = int(rng.choice([0, 32, 64]))
    sched = int(rng.integers(0, 3))
    try:
        ctx.set_tuning(threads, stage, 0, sched)
    except vox.VoxError:
        ctx.set_tuning(threads, 0, 0, sched)  # the staging window does not fit
    b0, b1 = ctx.sizes.bytes_per_face_out0, ctx.sizes.bytes_per_face_out1
    o0, o1 = dev_bytes(max(total, 1) * b0), dev_bytes(max(total, 1) * b1)
    offs = to_dev(np.zeros(m + 1, np.uint64))
    ctx.gen_mesh_batch(to_dev(np.asarray(coords, np.int32)), to_dev(np.asarray(masks, np.uint8)), m,
                       o0, o1 if b1 else None, total, offs, chunk_index_base=base)
    ctx.sync()
    tag = (n, kind, layout, cull, m, threads, stage, sched)
    assert np.array_equal(to_np(offs), woffs), tag
    assert np.array_equal(to_np(o0, total * b0), w0), tag
    if b1:
        assert np.array_equal(to_np(o1, total * b1), w1), tag
    ctx.close()


@pytest.mark.parametrize("n", [16, 32])
@pytest.mark.parametrize("kind", ["density4", "density1x", "refdensity"])
@pytest.mark.parametrize("halo", [0, 1])
def test_density_configs_fused_and_staged(vox, oracle, n, kind, halo):
    """Density generators at the table path's limits (4 octaves; lattice cells narrower
    than a block of x samples) through the fused launch (halos regenerated: per-sample
    table reads) and the staged-halo path (generation kernel, then meshing from the pool)."""
    rng = np.random.default_rng(77 + n + 3 * halo)
    cull = int(rng.integers(0, 2))
    cfg = gen_cfg(vox, kind, n, cull=cull)
    m = 20
    coords = [tuple(int(v) for v in rng.integers(-4, 4, 3)) for _ in range(m)]
    coords = list(dict.fromkeys(coords))  # distinct, so every chunk has one pool slot
    m = len(coords)
    masks = [int(v) for v in rng.integers(0, 64 if cull else 16, m)]
    w0, w1, woffs = oracle.gen_mesh_batch(cfg, coords, masks, 0)
    total = int(woffs[-1])
    ctx = ctx_for(vox, cfg)
    t = ctx.tuning()
    ctx.set_tuning(t.threads, t.stage_faces, 0, 2, 0, halo)
    o0, o1 = dev_bytes(max(total, 1) * 96), dev_bytes(max(total, 1) * 24)
    offs = to_dev(np.zeros(m + 1, np.uint64))
    ctx.gen_mesh_batch(to_dev(np.asarray(coords, np.int32)), to_dev(np.asarray(masks, np.uint8)), m,
                       o0, o1, total, offs)
    ctx.sync()
    assert np.array_equal(to_np(offs), woffs), (n, kind, halo)
    assert np.array_equal(to_np(o0, total * 96), w0), (n, kind, halo)
    assert np.array_equal(to_np(o1, total * 24), w1), (n, kind, halo)
    ctx.close()
