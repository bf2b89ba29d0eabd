"""Host-side logic without a GPU: workloads and neighbour masks, coordinate and camera
helpers of the streaming engine, and the rank sharding of the multi-process benchmark
(world size 2 over gloo)."""
import ctypes
import math
import os
import socket

import numpy as np
import pytest


def test_workloads_have_the_configured_shapes(vox):
    assert len(vox.workload("plain").coords) == 64
    hm = vox.workload("heightmap")
    assert len(hm.coords) == 1024 and hm.config().chunk_size == 16
    assert len(vox.workload("density").coords) == 4096
    st = vox.workload("stress")
    assert len(st.coords) == 2048 and st.isolated and set(st.masks()) == {0}


def test_neighbour_masks_follow_the_world_lookup(vox):
    coords = vox.grid_coords(range(3), [0], range(3))
    masks = dict(zip(coords, vox.neighbour_masks(coords)))
    assert masks[(1, 0, 1)] == 0b1111          # interior: all four lateral neighbours
    assert masks[(0, 0, 0)] == 0b1010          # only +x and +z exist
    assert vox.neighbour_masks([(0, 0, 0), (0, 1, 0)], full6=True) == [0b100000, 0b010000]


@pytest.mark.parametrize("pos,n,want", [((0.0, 0.0, 0.0), 32, (0, 0, 0)),
                                        ((-0.01, 31.99, 32.0), 32, (-1, 0, 1)),
                                        ((-33.0, 5.0, 70.5), 16, (-3, 0, 4))])
def test_world_to_chunk_floors_then_shifts(vox, pos, n, want):
    c = vox.lib().vox_world_to_chunk((ctypes.c_float * 3)(*pos), n)
    assert (c.x, c.y, c.z) == want  # Coord3DF::to_chunk_coord, src/coordinate.rs:33-38


def test_camera_matrix_sees_ahead_not_behind(vox, oracle):
    eye, d = vox.serving_camera(0.0)
    m = vox.camera_matrix(eye, d, zfar=500.0)
    planes = oracle.frustum_planes(np.array(m, np.float32))
    ahead = tuple(int(math.floor((e + 100 * v) / 16)) for e, v in zip(eye, d))
    behind = tuple(int(math.floor((e - 100 * v) / 16)) for e, v in zip(eye, d))
    assert oracle.frustum_contains(planes, ahead, 16)
    assert not oracle.frustum_contains(planes, behind, 16)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _shard_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import voxgpu
    for name in ("heightmap", "stress"):
        wl = bench.shard_workload(voxgpu.workload(name), rank, world)
        import torch
        t = torch.tensor([min(c[0] for c in wl.coords), wl.index_base], dtype=torch.int64)
        parts = [torch.zeros_like(t) for _ in range(world)]
        dist.all_gather(parts, t)
        ms = torch.tensor([float(rank + 1)])
        dist.all_reduce(ms, op=dist.ReduceOp.MAX)
        if rank == 0:
            out.put((name, [p.tolist() for p in parts], float(ms.item())))
    dist.destroy_process_group()


def test_bench_shards_are_disjoint_over_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got = {name: (parts, ms) for name, parts, ms in results}
    hm_parts, ms = got["heightmap"]
    assert hm_parts[0][0] != hm_parts[1][0]  # weak scaling: disjoint x ranges per rank
    st_parts, _ = got["stress"]
    assert st_parts[0][1] == 0 and st_parts[1][1] == 2048  # disjoint Bernoulli index ranges
    assert ms == 2.0  # the time reported is the maximum over ranks
