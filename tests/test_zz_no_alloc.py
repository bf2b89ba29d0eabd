"""vox_gen_mesh_batch_noalloc: the fused generation + meshing call for callers that cannot
allocate device memory (an engine or framework that owns every device allocation through
its own pool, or code that must not allocate once it is running).

The call takes the same inputs and outputs as vox_gen_mesh_batch but needs no context and
allocates nothing; its scratch is a static array inside the library. These tests call it
through the C ABI and require its output to equal, byte for byte, what the context-based
vox_gen_mesh_batch produces on the same batch, on two calls in a row (the second call
reuses the scratch the first one left behind). This file is collected last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import ctx_for, dev_bytes, to_dev, to_np

pytestmark = pytest.mark.gpu


def _noalloc(vox, cfg, d_coords, d_mask, n, o0, o1, cap, offs, index_base=0):
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    return vox.lib().vox_gen_mesh_batch_noalloc(
        ctypes.byref(cfg), ctypes.c_void_p(stream), d_coords.data_ptr(),
        None if d_mask is None else d_mask.data_ptr(), n, index_base, o0.data_ptr(),
        None if o1 is None else o1.data_ptr(), cap, offs.data_ptr())


@pytest.mark.parametrize("wlname,layout,sub", [("heightmap", 0, 1024), ("plain", 1, 64),
                                               ("stress", 0, 3)])
def test_noalloc_matches_context_entry_point(vox, wlname, layout, sub):
    wl = vox.workload(wlname)
    cfg = wl.config(layout=layout)
    coords = list(wl.coords[:sub])
    masks = None if wl.isolated else wl.masks()[:sub]
    n = len(coords)
    d_coords = to_dev(np.asarray(coords, np.int32))
    d_mask = None if masks is None else to_dev(np.asarray(masks, np.uint8))
    # reference result from the context-based entry point
    ctx = ctx_for(vox, cfg)
    b0, b1 = ctx.sizes.bytes_per_face_out0, ctx.sizes.bytes_per_face_out1
    cap = ctx.sizes.max_faces_per_chunk * n
    r0, r1 = dev_bytes(cap * b0), dev_bytes(max(cap * b1, 16))
    roffs = to_dev(np.zeros(n + 1, np.uint64))
    ctx.gen_mesh_batch(d_coords, d_mask, n, r0, r1 if b1 else None, cap, roffs)
    ctx.sync()
    want_offs = to_np(roffs)
    total = int(want_offs[n])
    want0 = to_np(r0, total * b0)
    want1 = to_np(r1, total * b1) if b1 else None
    ctx.close()
    # two calls in a row through the no-allocation entry point
    for call in range(2):
        o0, o1 = dev_bytes(cap * b0, fill=0x3C), dev_bytes(max(cap * b1, 16), fill=0x3C)
        offs = to_dev(np.zeros(n + 1, np.uint64))
        st = _noalloc(vox, cfg, d_coords, d_mask, n, o0, o1 if b1 else None, cap, offs,
                      wl.index_base)
        assert st == vox.VOX_OK, (call, st)
        assert np.array_equal(to_np(offs), want_offs), call
        assert np.array_equal(to_np(o0, total * b0), want0), call
        if b1:
            assert np.array_equal(to_np(o1, total * b1), want1), call


def test_noalloc_rejects_batches_beyond_its_maximum(vox):
    wl = vox.workload("heightmap")
    cfg = wl.config()
    d_coords = to_dev(np.zeros((16385, 3), np.int32))
    o = dev_bytes(1024)
    offs = to_dev(np.zeros(16386, np.uint64))
    st = _noalloc(vox, cfg, d_coords, None, 16385, o, o, 1, offs)
    assert st == vox.VOX_ERR_INVALID


def test_noalloc_reports_a_short_output(vox):
    wl = vox.workload("plain")
    cfg = wl.config()
    coords = list(wl.coords[:8])
    masks = vox.neighbour_masks(coords)
    d_coords = to_dev(np.asarray(coords, np.int32))
    d_mask = to_dev(np.asarray(masks, np.uint8))
    o0, o1 = dev_bytes(100 * 96), dev_bytes(100 * 24)
    offs = to_dev(np.zeros(9, np.uint64))
    st = _noalloc(vox, cfg, d_coords, d_mask, 8, o0, o1, 100, offs)
    assert st == vox.VOX_ERR_CAPACITY
    assert int(to_np(offs)[8]) > 100  # the required size is still returned
