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


def test_noalloc_full_state_array(vox):
    """A call of exactly 16384 chunks uses every look-back state of the static array: the
    face offsets must equal the context entry point's (8^3 chunks, no output written)."""
    cfg = vox.make_config(chunk_size=8, octaves=1, seed=42, frequency=1 / 64, amplitude=12.0,
                          base_height=4.0)
    n = 16384
    coords = vox.grid_coords(range(-64, 64), range(-1, 1), range(-64, 0))
    assert len(coords) == n
    d_coords = to_dev(np.asarray(coords, np.int32))
    ctx = ctx_for(vox, cfg)
    roffs = to_dev(np.zeros(n + 1, np.uint64))
    ctx.gen_mesh_batch(d_coords, None, n, None, None, 0, roffs)
    assert ctx.sync(raise_on_error=False) == vox.VOX_ERR_CAPACITY  # nothing fits in 0 faces
    want = to_np(roffs)
    ctx.close()
    assert int(want[n]) > 0
    for call in range(2):
        offs = to_dev(np.zeros(n + 1, np.uint64))
        st = _noalloc_raw(vox, cfg, d_coords.data_ptr(), None, n, None, None, 0, offs.data_ptr())
        assert st == vox.VOX_ERR_CAPACITY, (call, st)
        assert np.array_equal(to_np(offs), want), call


def _noalloc_raw(vox, cfg, coords, mask, n, out0, out1, cap, offs, stream=None):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    return vox.lib().vox_gen_mesh_batch_noalloc(ctypes.byref(cfg), ctypes.c_void_p(stream),
                                                coords, mask, n, 0, out0, out1, cap, offs)


def test_noalloc_rejects_misaligned_or_missing_outputs(vox):
    cfg = vox.workload("plain").config()
    d_coords = to_dev(np.zeros((4, 3), np.int32))
    o = dev_bytes(1 << 16)
    offs = to_dev(np.zeros(5, np.uint64))
    p = o.data_ptr()
    assert _noalloc_raw(vox, cfg, d_coords.data_ptr(), None, 4, p + 4, p, 8, offs.data_ptr()) \
        == vox.VOX_ERR_INVALID
    assert _noalloc_raw(vox, cfg, d_coords.data_ptr(), None, 4, p, p + 8, 8, offs.data_ptr()) \
        == vox.VOX_ERR_INVALID
    assert _noalloc_raw(vox, cfg, d_coords.data_ptr(), None, 4, None, p, 8, offs.data_ptr()) \
        == vox.VOX_ERR_INVALID
    assert _noalloc_raw(vox, cfg, d_coords.data_ptr(), None, 4, p, None, 8, offs.data_ptr()) \
        == vox.VOX_ERR_INVALID


def test_noalloc_refuses_a_capturing_stream(vox):
    """The call is synchronous: on a stream under capture it returns VOX_ERR_INVALID and
    queues nothing, and the capture stays valid."""
    import torch
    cfg = vox.workload("plain").config()
    d_coords = to_dev(np.zeros((4, 3), np.int32))
    o0, o1 = dev_bytes(1 << 16), dev_bytes(1 << 16)
    offs = to_dev(np.zeros(5, np.uint64))
    marker = torch.zeros(4, dtype=torch.float32, device="cuda")
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        g.capture_begin()
        try:
            st = _noalloc_raw(vox, cfg, d_coords.data_ptr(), None, 4, o0.data_ptr(),
                              o1.data_ptr(), 8, offs.data_ptr(), stream=side.cuda_stream)
            marker.add_(1.0)  # the capture keeps one node of its own
        finally:
            g.capture_end()
    assert st == vox.VOX_ERR_INVALID
    g.replay()
    torch.cuda.synchronize()
    assert marker.cpu().tolist() == [1.0] * 4
