"""Helpers of the GPU tests: device buffers through torch, contexts on torch's stream,
and one-call wrappers that run a path on the device and bring the bytes back."""
import numpy as np


def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    return torch


def ctx_for(vox, cfg):
    """A context on torch's current stream. torch's default stream has the handle 0, which
    the C ABI reads as "create a stream of your own"; pass the legacy default stream
    (cudaStreamLegacy, handle 1) instead, so that the context's work and the tests' torch
    work on the default stream stay in one order."""
    torch = torch_cuda()
    return vox.Context(cfg, stream=torch.cuda.current_stream().cuda_stream or 1)


def to_dev(a, dtype=None):
    torch = torch_cuda()
    a = np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype=dtype))
    return torch.from_numpy(a.copy()).cuda()


def dev_bytes(nbytes, fill=None):
    torch = torch_cuda()
    n = max(int(nbytes), 16)
    t = torch.empty(n, dtype=torch.uint8, device="cuda")
    if fill is not None:
        t.fill_(fill)
    return t


def to_np(t, nbytes=None):
    torch = torch_cuda()
    torch.cuda.synchronize()
    a = t.cpu().numpy()
    if nbytes is not None:
        a = a.view(np.uint8)[:nbytes]
    return a


def use_schedule(ctx, schedule):
    """Keeps the context's launch shape and selects a schedule (None: leave it)."""
    if schedule is not None:
        t = ctx.tuning()
        ctx.set_tuning(t.threads, t.stage_faces, t.ctas_per_sm, schedule)


def gpu_gen_mesh(vox, cfg, coords, masks=None, index_base=0, cap=None, expect_status=None,
                 schedule=None):
    """Runs vox_gen_mesh_batch; returns (out0 bytes, out1 bytes, offsets, status)."""
    ctx = ctx_for(vox, cfg)
    use_schedule(ctx, schedule)
    n = len(coords)
    d_coords = to_dev(np.asarray(coords, np.int32).reshape(-1, 3))
    d_mask = None if masks is None else to_dev(np.asarray(masks, np.uint8))
    b0 = ctx.sizes.bytes_per_face_out0
    b1 = ctx.sizes.bytes_per_face_out1
    if cap is None:
        cap = ctx.sizes.max_faces_per_chunk * n
    o0 = dev_bytes(cap * b0, fill=0xAB)
    o1 = dev_bytes(cap * b1, fill=0xCD)
    offs = to_dev(np.zeros(n + 1, np.uint64))
    ctx.gen_mesh_batch(d_coords, d_mask, n, o0, o1 if b1 else None, cap, offs,
                       chunk_index_base=index_base)
    st = ctx.sync(raise_on_error=expect_status is None)
    offsets = to_np(offs)
    total = int(offsets[n])
    w = min(total, cap)
    out0 = to_np(o0, w * b0)
    out1 = to_np(o1, w * b1) if b1 else np.zeros(0, np.uint8)
    ctx.close()
    return out0, out1, offsets, st


def gpu_generate(vox, cfg, coords, index_base=0):
    ctx = ctx_for(vox, cfg)
    n = len(coords)
    words = ctx.sizes.occ_words_per_chunk
    d_coords = to_dev(np.asarray(coords, np.int32).reshape(-1, 3))
    occ = dev_bytes(n * words * 4)
    ctx.generate(d_coords, n, occ, chunk_index_base=index_base)
    ctx.sync()
    out = to_np(occ, n * words * 4).view(np.uint32).reshape(n, words)
    ctx.close()
    return out


class Pinned:
    """A page-locked host buffer from vox_host_alloc with a numpy view."""

    def __init__(self, vox, nbytes):
        import ctypes
        self._lib = vox.lib()
        p = ctypes.c_void_p()
        assert self._lib.vox_host_alloc(max(16, int(nbytes)), ctypes.byref(p)) == 0
        self.ptr = p.value
        self.nbytes = int(nbytes)
        self.a = np.ctypeslib.as_array((ctypes.c_uint8 * max(16, int(nbytes))).from_address(self.ptr))

    def view(self, dtype):
        return self.a[:self.nbytes].view(dtype)

    def free(self):
        if self.ptr:
            self._lib.vox_host_free(self.ptr)
            self.ptr = None
