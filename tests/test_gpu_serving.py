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
