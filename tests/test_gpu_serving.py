"""The chunk streaming engine (include/voxgpu_serve.h) on the GPU: continuous batching,
the device mesh cache, LRU eviction under a byte budget, latency statistics, and the
invariance of every chunk's mesh under batching (alone == in the mix)."""
import ctypes

import numpy as np
import pytest

from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu


def run_frames(vox, server, frames, dt=1.0 / 60):
    for k in range(frames):
        eye, d = vox.serving_camera(k * dt)
        m = vox.camera_matrix(eye, d, zfar=500.0)
        server.frame(m, eye)
    server.drain()


class _DeviceBytes:
    """A raw device pointer seen through the CUDA array interface (a torch view)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "|u1", "data": (ptr, False),
                                         "version": 2}


def fetch(ptr, nbytes):
    """Copies nbytes from a raw device pointer to host memory."""
    torch = torch_cuda()
    torch.cuda.synchronize()
    if nbytes == 0:
        return np.zeros(0, np.uint8)
    return torch.as_tensor(_DeviceBytes(ptr, nbytes), device="cuda").cpu().numpy()


def test_camera_and_world_to_chunk(vox):
    c = vox.lib().vox_world_to_chunk((ctypes.c_float * 3)(-0.5, 15.9, 16.0), 16)
    assert (c.x, c.y, c.z) == (-1, 0, 1)
    m = np.array(vox.camera_matrix((0, 0, 0), (0, 0, -1)), np.float32)
    assert np.isfinite(m).all()


def test_serving_meshes_equal_alone_and_complete(vox, oracle):
    wl = vox.workload("heightmap")
    cfg = wl.config()
    server = vox.Server(cfg, view_radius=12, max_batch=32, slots=3)
    run_frames(vox, server, 90)
    st = server.stats()
    assert st.requested > 100
    assert st.completed == st.requested and st.pending == 0
    assert 0 < st.latency_p50_ms <= st.latency_p99_ms <= st.latency_max_ms
    # every resident chunk's mesh equals the chunk meshed alone with all lateral
    # neighbours present, on the GPU and in the oracle
    eye, _ = vox.serving_camera(90 / 60)
    centre = vox.lib().vox_world_to_chunk((ctypes.c_float * 3)(*eye), 16)
    checked = 0
    for dz in range(-12, 13, 3):
        for dx in range(-12, 13, 3):
            c = (centre.x + dx, 0, centre.z + dz)
            got = server.lookup(c)
            if got is None:
                continue
            p0, p1, faces = got
            w0, w1, woffs = oracle.gen_mesh_batch(cfg, [c], [0x0F])
            assert faces == int(woffs[-1])
            assert np.array_equal(fetch(p0, faces * 96), w0)
            assert np.array_equal(fetch(p1, faces * 24), w1)
            checked += 1
    assert checked >= 5
    server.close()


def test_serving_evicts_lru_under_budget(vox):
    wl = vox.workload("heightmap")
    cfg = wl.config()
    budget = 24 << 20
    server = vox.Server(cfg, view_radius=12, max_batch=16, slots=2, cache_budget_bytes=budget)
    run_frames(vox, server, 240)
    st = server.stats()
    assert st.evicted > 0
    assert st.cache_bytes <= budget
    assert st.completed >= st.requested - st.pending
    server.close()


def test_submit_poll_wait_by_request_id(vox, oracle):
    """Explicit requests: ids are stable per chunk, wait returns when resident, the mesh is
    the chunk's final mesh, and unknown ids are reported as such."""
    wl = vox.workload("heightmap")
    cfg = wl.config()
    server = vox.Server(cfg, view_radius=4, max_batch=8, slots=2)
    coords = [(3, 0, -2), (4, 0, -2), (-7, 0, 9), (0, 0, 0), (11, 0, 5)]
    ids = server.submit(coords)
    assert len(set(ids)) == len(coords) and all(i > 0 for i in ids)
    assert server.submit(coords[:2]) == ids[:2]  # the same chunks keep their ids
    assert server.poll(10 ** 9) == vox.VOX_REQ_UNKNOWN
    assert server.wait(10 ** 9, 1.0) == vox.VOX_ERR_INVALID
    for c, i in zip(coords, ids):
        assert server.poll(i) in (vox.VOX_REQ_PENDING, vox.VOX_REQ_RESIDENT)
        assert server.wait(i, 30.0) == vox.VOX_OK
        assert server.poll(i) == vox.VOX_REQ_RESIDENT
        p0, p1, faces = server.lookup(c)
        # the engine generates every lateral halo: the chunk's mesh with all four present
        w0, w1, woffs = oracle.gen_mesh_batch(cfg, [c], [0x0F])
        assert faces == int(woffs[-1])
        assert np.array_equal(fetch(p0, faces * 96), w0)
        assert np.array_equal(fetch(p1, faces * 24), w1)
    st = server.stats()
    assert st.requested == len(coords) and st.completed == len(coords)
    server.close()


def test_cancel_withdraws_queued_and_in_flight_requests(vox, oracle):
    """A cancelled request never becomes resident, whether it was still queued or its batch
    was already on the GPU; the other requests complete with their final meshes, and the
    chunk can be requested again."""
    wl = vox.workload("heightmap")
    cfg = wl.config()
    server = vox.Server(cfg, view_radius=4, max_batch=8, slots=1)
    coords = [(x, 0, z) for z in range(6) for x in range(6)]
    ids = server.submit(coords)  # the 8 nearest (to the origin) go to the GPU at once
    first, far = coords.index((0, 0, 0)), coords.index((5, 0, 5))
    assert server.cancel(ids[first]) == vox.VOX_OK  # in flight
    assert server.cancel(ids[far]) == vox.VOX_OK    # queued
    assert server.cancel(ids[far]) == vox.VOX_ERR_INVALID
    assert server.cancel(10 ** 9) == vox.VOX_ERR_INVALID
    server.drain()
    assert server.poll(ids[first]) == vox.VOX_REQ_UNKNOWN
    assert server.poll(ids[far]) == vox.VOX_REQ_UNKNOWN
    assert server.lookup((0, 0, 0)) is None and server.lookup((5, 0, 5)) is None
    st = server.stats()
    assert st.cancelled == 2 and st.pending == 0
    assert st.resident == len(coords) - 2 and st.completed == len(coords) - 2
    done = coords.index((1, 0, 1))
    assert server.cancel(ids[done]) == vox.VOX_ERR_INVALID  # resident: nothing to withdraw
    # requested again: a new id, and the mesh of the chunk alone
    again = server.submit([(0, 0, 0)])[0]
    assert again not in ids
    assert server.wait(again, 30.0) == vox.VOX_OK
    for c in ((0, 0, 0), (1, 0, 1)):
        p0, p1, faces = server.lookup(c)
        w0, w1, woffs = oracle.gen_mesh_batch(cfg, [c], [0x0F])
        assert faces == int(woffs[-1])
        assert np.array_equal(fetch(p0, faces * 96), w0)
        assert np.array_equal(fetch(p1, faces * 24), w1)
    server.close()


def test_cache_budget_exhaustion_reports_oom_and_recovers(vox):
    """A cache budget below one batch's reservation (an injected allocation failure of the
    chunk cache): nothing is launched, wait and drain report VOX_ERR_OOM instead of
    spinning, and withdrawing the requests leaves a usable, empty engine."""
    wl = vox.workload("heightmap")
    cfg = wl.config()
    server = vox.Server(cfg, view_radius=4, max_batch=4, slots=2, cache_budget_bytes=64 << 10)
    ids = server.submit([(0, 0, 0), (1, 0, 0), (2, 0, 0)])
    assert server.wait(ids[0], 5.0) == vox.VOX_ERR_OOM
    with pytest.raises(vox.VoxError):
        server.drain()
    for i in ids:
        assert server.cancel(i) == vox.VOX_OK
    server.drain()
    st = server.stats()
    assert st.launches == 0 and st.pending == 0 and st.resident == 0 and st.cancelled == 3
    server.close()


LATERAL = ((-1, 0), (1, 0), (0, -1), (0, 1))


def oracle_mesh_with(oracle, cfg, c, present):
    """The oracle's mesh of chunk c with the lateral neighbours in `present` loaded and the
    others absent (their border faces emitted, src/chunk.rs:102-107)."""
    adj = []
    for dx, dz in LATERAL:
        q = (c[0] + dx, c[1], c[2] + dz)
        adj.append(oracle.generate_cubes(cfg, q, 0) if q in present else None)
    return oracle.mesh_chunk(cfg, c, oracle.generate_cubes(cfg, c, 0), adj)


def check_resident_against_oracle(server, oracle, cfg, coords):
    """Every resident chunk of `coords` has the mesh the reference builds with its resident
    lateral neighbours; returns the resident set."""
    present = {c for c in coords if server.lookup(c) is not None}
    for c in present:
        p0, p1, faces = server.lookup(c)
        w0, w1, cnt = oracle_mesh_with(oracle, cfg, c, present)
        assert faces == cnt, (c, faces, cnt)
        assert np.array_equal(fetch(p0, faces * 96), w0), c
        assert np.array_equal(fetch(p1, faces * 24), w1), c
    return present


def test_neighbour_rebuild_remeshes_when_a_neighbour_arrives(vox, oracle):
    """neighbour_rebuild = 1 (src/chunk_builder.rs:89-112, 269-300, 310-332): a chunk meshed
    before its neighbour arrives has its border faces; once the neighbour is resident the
    chunk is remeshed from its cached occupancy and equals the oracle with the neighbour."""
    cfg = vox.workload("heightmap").config()
    server = vox.Server(cfg, view_radius=4, max_batch=8, slots=2, neighbour_rebuild=True)
    a, b = (3, 0, -2), (4, 0, -2)
    ida = server.submit([a])[0]
    assert server.wait(ida, 30.0) == vox.VOX_OK
    server.drain()
    p0, p1, faces = server.lookup(a)
    w0, w1, cnt = oracle_mesh_with(oracle, cfg, a, set())
    alone = faces
    assert faces == cnt and np.array_equal(fetch(p0, faces * 96), w0)
    idb = server.submit([b])[0]
    assert server.wait(idb, 30.0) == vox.VOX_OK
    server.drain()
    check_resident_against_oracle(server, oracle, cfg, [a, b])
    assert server.lookup(a)[2] < alone  # the shared border is culled now
    st = server.stats()
    assert st.rebuilt >= 1 and st.rebuild_launches >= 1 and st.completed == 2
    server.close()


def test_neighbour_rebuild_converges_in_any_arrival_order(vox, oracle):
    """Chunks of an 8 x 8 area requested in random waves, some batches in flight together,
    a few requests cancelled: once drained, every resident chunk equals the oracle with its
    resident neighbours."""
    cfg = vox.workload("heightmap").config()
    rng = np.random.default_rng(3)
    coords = [(x, 0, z) for z in range(-4, 4) for x in range(-4, 4)]
    order = [coords[i] for i in rng.permutation(len(coords))]
    server = vox.Server(cfg, view_radius=4, max_batch=5, slots=3, neighbour_rebuild=True)
    cancelled = set()
    for k in range(0, len(order), 9):
        ids = server.submit(order[k:k + 9])
        if k == 18:
            server.cancel(ids[0])
            cancelled.add(order[k])
    server.drain()
    present = check_resident_against_oracle(server, oracle, cfg, coords)
    assert present == set(coords) - cancelled
    server.close()


def test_neighbour_rebuild_after_eviction(vox, oracle):
    """A cache budget that holds about 20 chunks: evictions free occupancy slots and queue
    rebuilds of the neighbours that saw the evicted chunk; after draining, the resident
    chunks still equal the oracle with their resident neighbours."""
    cfg = vox.workload("heightmap").config()
    per_chunk = 4 * 16 * 16 * 120
    server = vox.Server(cfg, view_radius=4, max_batch=4, slots=2, neighbour_rebuild=True,
                        cache_budget_bytes=20 * per_chunk)
    coords = [(x, 0, z) for z in range(6) for x in range(6)]
    for k in range(0, len(coords), 4):
        server.submit(coords[k:k + 4])
        server.drain()
    st = server.stats()
    assert st.evicted > 0
    present = check_resident_against_oracle(server, oracle, cfg, coords)
    assert 0 < len(present) <= 20
    server.close()


def test_neighbour_rebuild_with_the_camera(vox, oracle):
    """The camera-driven loop in neighbour-rebuild mode: requests, batches and rebuilds
    interleave over 60 frames; drained, the resident chunks equal the oracle."""
    cfg = vox.workload("heightmap").config()
    server = vox.Server(cfg, view_radius=8, max_batch=32, slots=3, neighbour_rebuild=True)
    run_frames(vox, server, 60)
    st = server.stats()
    assert st.completed == st.requested and st.rebuilt > 0
    eye, _ = vox.serving_camera(60 / 60)
    centre = vox.lib().vox_world_to_chunk((ctypes.c_float * 3)(*eye), 16)
    area = [(centre.x + dx, 0, centre.z + dz) for dz in range(-9, 10) for dx in range(-9, 10)]
    present = check_resident_against_oracle(server, oracle, cfg, area)
    assert len(present) > 20
    server.close()


def test_latency_since_a_time_and_stats(vox):
    """vox_serve_latency over the requests issued after a time: the steady-state figures
    the benchmark reports next to the overall ones."""
    cfg = vox.workload("heightmap").config()
    server = vox.Server(cfg, view_radius=8, max_batch=32, slots=3)
    t0 = vox.Server.now()
    run_frames(vox, server, 120)
    p50, p99, mx, cnt = server.latency()
    st = server.stats()
    assert cnt == st.completed and p99 == pytest.approx(st.latency_p99_ms)
    later = server.latency(t0 + 0.5)
    assert later[3] <= cnt
    assert server.latency(1e300)[3] == 0
    server.close()
