"""A whole batch of chunks resident on the device, meshed by one call or by replays of one
captured graph, with the context's (optionally autotuned) launch shape and output slab.

This is the host-side loop the reference runs once per tick (the pool dispatch of
src/chunk_builder.rs:69-87, Chunk::new + create_mesh per chunk), for a fixed batch whose
buffers stay in device memory: the coordinates and neighbour masks are uploaded once, the
output is sized from a counting pass, and every step replays the same launches. Device
memory comes from torch (plumbing only); every launch goes through the C ABI.
"""
from __future__ import annotations

from . import VOX_OK, VOX_ERR_CAPACITY, VoxError


class BatchRun:
    """n chunks (coords, masks) meshed into device buffers sized for the whole batch.

    After construction: `offsets` (n + 1 int64 on the device, chunk i's first face and the
    total), `out0` / `out1` (uint8 device tensors of total * bytes-per-face), `total_faces`,
    `tuning` (the context's launch shape as a dict) and, with graph=True, one captured graph
    holding every slab launch of the batch."""

    def __init__(self, ctx, coords, masks=None, index_base: int = 0, autotune: bool = False,
                 tune_iters: int = 3, graph: bool = True):
        import torch
        self.ctx = ctx
        self.n = n = len(coords)
        self.index_base = index_base
        self.d_coords = torch.tensor(list(coords), dtype=torch.int32, device="cuda").reshape(n, 3)
        self.d_mask = (None if masks is None
                       else torch.tensor(list(masks), dtype=torch.uint8, device="cuda"))
        self.offsets = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
        self.b0 = ctx.sizes.bytes_per_face_out0
        self.b1 = ctx.sizes.bytes_per_face_out1
        torch.cuda.synchronize()
        # counting pass: with no output room the offsets are still complete
        ctx.gen_mesh_batch(self.d_coords, self.d_mask, n, None, None, 0, self.offsets,
                           chunk_index_base=index_base)
        st = ctx.sync(raise_on_error=False)
        if st not in (VOX_OK, VOX_ERR_CAPACITY):
            raise VoxError(st, "counting pass")
        self.total_faces = int(self.offsets[n].item())
        self.cap = max(self.total_faces, 1)
        self.out0 = torch.empty(self.cap * self.b0 + 16, dtype=torch.uint8, device="cuda")
        self.out1 = (torch.empty(self.cap * self.b1 + 16, dtype=torch.uint8, device="cuda")
                     if self.b1 else None)
        self.autotuned = False
        if autotune:
            ctx.autotune(self.d_coords, self.d_mask, n, self.out0, self.out1, self.cap,
                         self.offsets, chunk_index_base=index_base, iters=tune_iters)
            self.autotuned = True
        t = ctx.tuning()
        self.tuning = t.as_dict() | {"autotuned": self.autotuned}
        slab = t.slab_chunks if 0 < t.slab_chunks < n else n
        self.launches_per_step = (n + slab - 1) // slab
        if t.halo_staging:
            # staged halos: coordinate map (with the identity slots), neighbour lookup,
            # generation of the batch and (with neighbour masks) of the halo planes outside it
            self.launches_per_step += 3 + (1 if masks is not None else 0)
        self.graph = (ctx.capture_graph(self.d_coords, self.d_mask, n, self.out0, self.out1,
                                        self.cap, self.offsets, chunk_index_base=index_base)
                      if graph else None)

    def launch(self):
        """One pass over the batch (asynchronous on the context's stream)."""
        if self.graph is not None:
            self.graph.launch()
        else:
            self.ctx.gen_mesh_batch(self.d_coords, self.d_mask, self.n, self.out0, self.out1,
                                    self.cap, self.offsets, chunk_index_base=self.index_base)

    def host_offsets(self):
        """The n + 1 face offsets as a numpy uint64 array (synchronises)."""
        import numpy as np
        import torch
        torch.cuda.synchronize()
        return self.offsets.cpu().numpy().view(np.uint64)

    def chunk_bytes(self, i: int):
        """Chunk i's out0 and out1 bytes, copied to host numpy arrays (synchronises)."""
        import numpy as np
        import torch
        torch.cuda.synchronize()
        lo, hi = (int(v) for v in self.offsets[i:i + 2].cpu())
        o0 = self.out0[lo * self.b0:hi * self.b0].cpu().numpy()
        o1 = (self.out1[lo * self.b1:hi * self.b1].cpu().numpy() if self.b1
              else np.zeros(0, np.uint8))
        return o0, o1

    def close(self):
        """Destroys the captured graph and drops the output buffers."""
        if self.graph is not None:
            self.graph.close()
            self.graph = None
        self.out0 = self.out1 = None
