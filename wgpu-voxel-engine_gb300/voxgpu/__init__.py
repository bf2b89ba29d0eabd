"""voxgpu — Python bindings of the C ABI in include/voxgpu.h (ctypes).

The product is the CUDA library ``libvoxgpu.so`` built in this directory; these
bindings only marshal arguments. There is no CPU fallback: if the library is missing
or no GPU is visible, calls raise.

Device buffers are passed as integers (raw device pointers) or as objects with a
``data_ptr()`` method (torch tensors), so PyTorch can provide device memory and
streams without appearing in any signature.
"""
from __future__ import annotations

import ctypes
import os
import sys
import weakref
from dataclasses import dataclass

from . import _build

__all__ = [
    "VOX_OK", "VOX_ERR_INVALID", "VOX_ERR_OOM", "VOX_ERR_CUDA", "VOX_ERR_TIMEOUT",
    "VOX_ERR_CAPACITY", "VOX_ERR_NO_DEVICE", "GEN_HEIGHTMAP", "GEN_DENSITY", "GEN_BERNOULLI",
    "CULL_REFERENCE", "CULL_FULL6", "LAYOUT_VERTEX", "LAYOUT_INSTANCED", "SCHEDULE_LOOKBACK",
    "SCHEDULE_PHASED", "SCHEDULE_OVERLAP", "VOX_REQ_UNKNOWN", "VOX_REQ_PENDING",
    "VOX_REQ_RESIDENT", "GRASS_TEXTURES", "ChunkCoord", "Generator", "Config", "Sizes",
    "Tuning", "ServeConfig", "ServeStats", "VoxError", "lib", "make_config", "query_sizes",
    "frustum_planes", "Context", "Graph", "camera_matrix", "Server", "serving_camera",
    "grid_coords", "neighbour_masks", "Workload", "workload",
]

VOX_OK, VOX_ERR_INVALID, VOX_ERR_OOM, VOX_ERR_CUDA = 0, 1, 2, 3
VOX_ERR_TIMEOUT, VOX_ERR_CAPACITY, VOX_ERR_NO_DEVICE = 4, 5, 6
GEN_HEIGHTMAP, GEN_DENSITY, GEN_BERNOULLI = 0, 1, 2
CULL_REFERENCE, CULL_FULL6 = 0, 1
LAYOUT_VERTEX, LAYOUT_INSTANCED = 0, 1
SCHEDULE_LOOKBACK, SCHEDULE_PHASED, SCHEDULE_OVERLAP = 0, 1, 2
VOX_REQ_UNKNOWN, VOX_REQ_PENDING, VOX_REQ_RESIDENT = 0, 1, 2
# TEXTURE_INDEX_LIST row of GRASS (src/texture.rs:240-243), by face slot L R Bk F Up Down.
GRASS_TEXTURES = (0, 0, 0, 0, 2, 1)


class ChunkCoord(ctypes.Structure):
    """ChunkCoord3D (src/coordinate.rs:146-151)."""
    _fields_ = [("x", ctypes.c_int32), ("y", ctypes.c_int32), ("z", ctypes.c_int32)]


class Generator(ctypes.Structure):
    """vox_generator: the terrain generator (heightmap, density or Bernoulli) and its
    noise parameters."""
    _fields_ = [
        ("kind", ctypes.c_int32), ("octaves", ctypes.c_int32), ("seed", ctypes.c_uint64),
        ("frequency", ctypes.c_float), ("lacunarity", ctypes.c_float), ("gain", ctypes.c_float),
        ("amplitude", ctypes.c_float), ("base_height", ctypes.c_float), ("y_ref", ctypes.c_float),
        ("y_scale", ctypes.c_float), ("solid_below_zero", ctypes.c_int32),
    ]


class Config(ctypes.Structure):
    """vox_config: chunk size, cull mode, output layout, texture slots and generator."""
    _fields_ = [
        ("chunk_size", ctypes.c_int32), ("cull_mode", ctypes.c_int32), ("layout", ctypes.c_int32),
        ("texture_index", ctypes.c_uint32 * 6), ("gen", Generator),
    ]


class Sizes(ctypes.Structure):
    """vox_sizes: occupancy words per chunk, bytes per face of each output, faces per chunk
    at most."""
    _fields_ = [
        ("occ_words_per_chunk", ctypes.c_uint32), ("bytes_per_face_out0", ctypes.c_uint32),
        ("bytes_per_face_out1", ctypes.c_uint32), ("max_faces_per_chunk", ctypes.c_uint32),
    ]


class Tuning(ctypes.Structure):
    """vox_tuning: launch shape, schedule, output slab and halo staging of a context."""
    _fields_ = [("threads", ctypes.c_int32), ("stage_faces", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("schedule", ctypes.c_int32),
                ("slab_chunks", ctypes.c_int32), ("halo_staging", ctypes.c_int32)]

    def as_dict(self):
        """The tuning with the schedule and the halo staging by name."""
        return {"threads": self.threads, "stage_faces": self.stage_faces,
                "ctas_per_sm": self.ctas_per_sm,
                "schedule": {SCHEDULE_PHASED: "phased", SCHEDULE_OVERLAP: "overlap"}.get(
                    self.schedule, "lookback"),
                "slab_chunks": self.slab_chunks,
                "halo": "pool" if self.halo_staging else "regenerated"}


class ServeConfig(ctypes.Structure):
    """vox_serve_config: the streaming engine's chunk config, view disk, batching and cache
    budget."""
    _fields_ = [("chunk", Config), ("view_radius", ctypes.c_int32), ("y_min", ctypes.c_int32),
                ("y_max", ctypes.c_int32), ("max_batch", ctypes.c_int32),
                ("slots", ctypes.c_int32), ("cache_budget_bytes", ctypes.c_uint64),
                ("neighbour_rebuild", ctypes.c_int32)]


class ServeStats(ctypes.Structure):
    """vox_serve_stats: the streaming engine's counters and request-to-mesh latency."""
    _fields_ = [("frames", ctypes.c_uint64), ("requested", ctypes.c_uint64),
                ("completed", ctypes.c_uint64), ("evicted", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("faces_resident", ctypes.c_uint64),
                ("cache_bytes", ctypes.c_uint64), ("resident", ctypes.c_uint64),
                ("pending", ctypes.c_uint64), ("latency_p50_ms", ctypes.c_double),
                ("latency_p99_ms", ctypes.c_double), ("latency_max_ms", ctypes.c_double),
                ("busy_s", ctypes.c_double), ("cancelled", ctypes.c_uint64),
                ("rebuilt", ctypes.c_uint64), ("rebuild_launches", ctypes.c_uint64)]

    def as_dict(self):
        """Every field by name."""
        return {k: getattr(self, k) for k, _ in self._fields_}


class VoxError(RuntimeError):
    """A non-zero status of a C ABI call (where the reference would panic), with the
    context's last error message."""

    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        msg = f"{what}: status {status}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


_LIB = None

# Exported functions: name -> (restype, argtypes).
_P = ctypes.c_void_p
_SIGS = {
    "vox_abi_version": (ctypes.c_int, []),
    "vox_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "vox_query_sizes": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(Sizes)]),
    "vox_ctx_create": (ctypes.c_int, [ctypes.POINTER(Config), _P, ctypes.POINTER(_P)]),
    "vox_ctx_destroy": (ctypes.c_int, [_P]),
    "vox_ctx_sync": (ctypes.c_int, [_P]),
    "vox_ctx_stream": (_P, [_P]),
    "vox_ctx_last_error": (ctypes.c_char_p, [_P]),
    "vox_generate": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_int64, _P]),
    "vox_generate_slots": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_int64, _P,
                                          ctypes.c_int32, _P]),
    "vox_occ_to_cubes": (ctypes.c_int, [_P, _P, ctypes.c_int32, _P]),
    "vox_cubes_to_occ": (ctypes.c_int, [_P, _P, ctypes.c_int32, _P]),
    "vox_mesh": (ctypes.c_int, [_P, _P, ctypes.POINTER(_P), ChunkCoord, _P, _P, ctypes.c_uint64,
                                _P]),
    "vox_mesh_batch": (ctypes.c_int, [_P, _P, ctypes.c_int32, _P, _P, _P, ctypes.c_int32, _P, _P,
                                      ctypes.c_uint64, _P]),
    "vox_gen_mesh_batch": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int64, _P, _P,
                                          ctypes.c_uint64, _P]),
    "vox_gen_mesh_host": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int64, _P, _P,
                                         ctypes.c_uint64, _P]),
    "vox_gen_mesh_batch_noalloc": (ctypes.c_int, [ctypes.POINTER(Config), _P, _P, _P,
                                                  ctypes.c_int32, ctypes.c_int64, _P, _P,
                                                  ctypes.c_uint64, _P]),
    "vox_frustum_planes": (ctypes.c_int, [_P, _P]),
    "vox_frustum_cull": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, _P]),
    "vox_raster": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32,
                                  _P, _P]),
    "vox_ctx_get_tuning": (ctypes.c_int, [_P, ctypes.POINTER(Tuning)]),
    "vox_ctx_set_tuning": (ctypes.c_int, [_P, ctypes.POINTER(Tuning)]),
    "vox_autotune": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int64, _P, _P,
                                    ctypes.c_uint64, _P, ctypes.c_int32, ctypes.POINTER(Tuning)]),
    "vox_selftest_lookback_timeout": (ctypes.c_int, [_P, ctypes.c_int32]),
    "vox_graph_capture": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int64, _P, _P,
                                         ctypes.c_uint64, _P, ctypes.POINTER(_P)]),
    "vox_graph_launch": (ctypes.c_int, [_P]),
    "vox_draw_list": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int32, _P, _P]),
    "vox_graph_destroy": (ctypes.c_int, [_P]),
    "vox_serve_create": (ctypes.c_int, [ctypes.POINTER(ServeConfig), ctypes.POINTER(_P)]),
    "vox_serve_destroy": (ctypes.c_int, [_P]),
    "vox_serve_now": (ctypes.c_double, []),
    "vox_serve_frame": (ctypes.c_int, [_P, _P, _P, ctypes.c_double]),
    "vox_serve_drain": (ctypes.c_int, [_P]),
    "vox_serve_submit": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_double, _P]),
    "vox_serve_poll": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int32)]),
    "vox_serve_wait": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_double]),
    "vox_serve_cancel": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "vox_serve_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(ServeStats)]),
    "vox_serve_latency": (ctypes.c_int, [_P, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_uint64)]),
    "vox_serve_lookup": (ctypes.c_int, [_P, ChunkCoord, ctypes.POINTER(_P), ctypes.POINTER(_P),
                                        ctypes.POINTER(ctypes.c_uint64)]),
    "vox_camera_global_matrix": (ctypes.c_int, [_P, _P, ctypes.c_float, ctypes.c_float,
                                                ctypes.c_float, ctypes.c_float, _P]),
    "vox_world_to_chunk": (ChunkCoord, [_P, ctypes.c_int32]),
    "vox_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(_P)]),
    "vox_host_free": (ctypes.c_int, [_P]),
}


def lib(build_if_missing: bool = False) -> ctypes.CDLL:
    """Loads libvoxgpu.so from this directory (raises if it was not built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
        _build.build_library()
    handle = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = handle
    return handle


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if isinstance(x, ctypes.Array) or isinstance(x, ctypes.Structure):
        return ctypes.addressof(x)
    if hasattr(x, "ctypes"):  # numpy array
        return int(x.ctypes.data)
    raise TypeError(f"cannot take a pointer of {type(x)!r}")


def make_config(chunk_size=32, cull_mode=CULL_REFERENCE, layout=LAYOUT_VERTEX, kind=GEN_HEIGHTMAP,
                octaves=1, seed=42, frequency=1.0 / 64, lacunarity=2.0, gain=0.5, amplitude=12.0,
                base_height=4.0, y_ref=0.0, y_scale=0.0, solid_below_zero=0,
                textures=GRASS_TEXTURES) -> Config:
    """A vox_config from keyword arguments (the generator's fields flattened)."""
    cfg = Config()
    cfg.chunk_size = chunk_size
    cfg.cull_mode = cull_mode
    cfg.layout = layout
    for i, t in enumerate(textures):
        cfg.texture_index[i] = t
    g = cfg.gen
    g.kind, g.octaves, g.seed = kind, octaves, seed
    g.frequency, g.lacunarity, g.gain = frequency, lacunarity, gain
    g.amplitude, g.base_height, g.y_ref, g.y_scale = amplitude, base_height, y_ref, y_scale
    g.solid_below_zero = solid_below_zero
    return cfg


def query_sizes(cfg: Config) -> Sizes:
    """vox_query_sizes: the buffer sizes a config needs."""
    s = Sizes()
    st = lib().vox_query_sizes(ctypes.byref(cfg), ctypes.byref(s))
    if st != VOX_OK:
        raise VoxError(st, "vox_query_sizes")
    return s


def frustum_planes(m_colmajor) -> list:
    """Frustum::matrix_to_planes (src/frustum_culling.rs:47-85) via the C ABI."""
    m = (ctypes.c_float * 16)(*[float(v) for v in m_colmajor])
    out = (ctypes.c_float * 24)()
    st = lib().vox_frustum_planes(ctypes.addressof(m), ctypes.addressof(out))
    if st != VOX_OK:
        raise VoxError(st, "vox_frustum_planes")
    return list(out)


class Context:
    """One vox_ctx (one config, one stream)."""

    def __init__(self, cfg: Config, stream: int | None = None):
        self.cfg = cfg
        self._lib = lib()
        h = _P()
        st = self._lib.vox_ctx_create(ctypes.byref(cfg), _P(stream or 0), ctypes.byref(h))
        if st != VOX_OK:
            raise VoxError(st, "vox_ctx_create")
        self._h = h
        self.sizes = query_sizes(cfg)
        self._graphs = weakref.WeakSet()

    def close(self):
        """vox_ctx_destroy, after the context's captured graphs."""
        if getattr(self, "_h", None):
            for g in list(getattr(self, "_graphs", ())):
                g.close()  # a graph needs its context
            self._lib.vox_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        # no CUDA calls while the interpreter shuts down: the runtime may be gone already
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def stream(self) -> int:
        """The context's CUDA stream (vox_ctx_stream)."""
        return int(self._lib.vox_ctx_stream(self._h) or 0)

    def _check(self, st: int, what: str):
        if st != VOX_OK:
            detail = (self._lib.vox_ctx_last_error(self._h) or b"").decode()
            raise VoxError(st, what, detail)

    def sync(self, raise_on_error: bool = True) -> int:
        """vox_ctx_sync: waits for the context's work and returns its latched status."""
        st = self._lib.vox_ctx_sync(self._h)
        if raise_on_error:
            self._check(st, "vox_ctx_sync")
        return st

    def generate(self, d_coords, n: int, d_occ, chunk_index_base: int = 0):
        """vox_generate (Chunk::new, src/chunk.rs:21-46): occupancy of n chunks."""
        self._check(self._lib.vox_generate(self._h, _ptr(d_coords), n, chunk_index_base,
                                           _ptr(d_occ)), "vox_generate")

    def generate_slots(self, d_coords, n: int, d_pool, pool_slots: int, d_slots,
                       chunk_index_base: int = 0):
        """vox_generate_slots: occupancy of n chunks into the given slots of a pool."""
        self._check(self._lib.vox_generate_slots(self._h, _ptr(d_coords), n, chunk_index_base,
                                                 _ptr(d_pool), pool_slots, _ptr(d_slots)),
                    "vox_generate_slots")

    def occ_to_cubes(self, d_occ, n: int, d_cubes):
        """vox_occ_to_cubes: occupancy to the reference's one byte per voxel (Vec<Cube>)."""
        self._check(self._lib.vox_occ_to_cubes(self._h, _ptr(d_occ), n, _ptr(d_cubes)),
                    "vox_occ_to_cubes")

    def cubes_to_occ(self, d_cubes, n: int, d_occ):
        """vox_cubes_to_occ: one byte per voxel back to occupancy."""
        self._check(self._lib.vox_cubes_to_occ(self._h, _ptr(d_cubes), n, _ptr(d_occ)),
                    "vox_cubes_to_occ")

    def mesh(self, d_occ, nbrs, coord, d_out0, d_out1, cap_faces: int, d_count):
        """vox_mesh (Chunk::create_mesh, src/chunk.rs:48-245): one chunk with explicit
        neighbour occupancy (None: absent)."""
        arr = (_P * 6)(*[_P(_ptr(b)) for b in (list(nbrs) + [None] * 6)[:6]])
        c = ChunkCoord(*coord)
        self._check(self._lib.vox_mesh(self._h, _ptr(d_occ), arr, c, _ptr(d_out0), _ptr(d_out1),
                                       cap_faces, _ptr(d_count)), "vox_mesh")

    def mesh_batch(self, d_pool, pool_slots: int, d_slots, d_nbr_slots, d_coords, n: int, d_out0,
                   d_out1, cap_faces: int, d_offsets):
        """vox_mesh_batch: a batch meshed from occupancy resident in a pool (the rebuild
        path)."""
        self._check(self._lib.vox_mesh_batch(self._h, _ptr(d_pool), pool_slots, _ptr(d_slots),
                                             _ptr(d_nbr_slots), _ptr(d_coords), n, _ptr(d_out0),
                                             _ptr(d_out1), cap_faces, _ptr(d_offsets)),
                    "vox_mesh_batch")

    def gen_mesh_batch(self, d_coords, d_nbr_mask, n: int, d_out0, d_out1, cap_faces: int,
                       d_offsets, chunk_index_base: int = 0):
        """vox_gen_mesh_batch: generation and meshing of a batch in the fused launch
        (Chunk::new + create_mesh per chunk, src/chunk_builder.rs:80-84), device buffers."""
        self._check(self._lib.vox_gen_mesh_batch(self._h, _ptr(d_coords), _ptr(d_nbr_mask), n,
                                                 chunk_index_base, _ptr(d_out0), _ptr(d_out1),
                                                 cap_faces, _ptr(d_offsets)),
                    "vox_gen_mesh_batch")

    def gen_mesh_host(self, h_coords, h_nbr_mask, n: int, h_out0, h_out1, cap_faces: int,
                      h_offsets, chunk_index_base: int = 0, raise_on_error: bool = True) -> int:
        """vox_gen_mesh_host: as gen_mesh_batch with host buffers (page-locked outputs are
        written in place); returns the status."""
        st = self._lib.vox_gen_mesh_host(self._h, _ptr(h_coords), _ptr(h_nbr_mask), n,
                                         chunk_index_base, _ptr(h_out0), _ptr(h_out1), cap_faces,
                                         _ptr(h_offsets))
        if raise_on_error:
            self._check(st, "vox_gen_mesh_host")
        return st

    def tuning(self) -> Tuning:
        """vox_ctx_get_tuning."""
        t = Tuning()
        self._check(self._lib.vox_ctx_get_tuning(self._h, ctypes.byref(t)), "vox_ctx_get_tuning")
        return t

    def set_tuning(self, threads: int, stage_faces: int, ctas_per_sm: int = 0,
                   schedule: int = 0, slab_chunks: int = 0, halo_staging: int = 0):
        """vox_ctx_set_tuning."""
        t = Tuning(threads, stage_faces, ctas_per_sm, schedule, slab_chunks, halo_staging)
        self._check(self._lib.vox_ctx_set_tuning(self._h, ctypes.byref(t)), "vox_ctx_set_tuning")

    def autotune(self, d_coords, d_nbr_mask, n: int, d_out0, d_out1, cap_faces: int, d_offsets,
                 chunk_index_base: int = 0, iters: int = 3) -> Tuning:
        """vox_autotune: times the candidate tunings on this batch and keeps the fastest."""
        t = Tuning()
        self._check(self._lib.vox_autotune(self._h, _ptr(d_coords), _ptr(d_nbr_mask), n,
                                           chunk_index_base, _ptr(d_out0), _ptr(d_out1),
                                           cap_faces, _ptr(d_offsets), iters, ctypes.byref(t)),
                    "vox_autotune")
        return t

    def selftest_lookback_timeout(self, spin_limit: int) -> int:
        """vox_selftest_lookback_timeout: a bounded device wait made to run out; returns the
        status (VOX_ERR_TIMEOUT)."""
        return self._lib.vox_selftest_lookback_timeout(self._h, spin_limit)

    def draw_list(self, planes, d_coords, d_offsets, n: int, d_draws, d_count):
        """vox_draw_list: indirect draw records of the visible chunks with faces."""
        p = (ctypes.c_float * 24)(*[float(v) for v in planes])
        self._check(self._lib.vox_draw_list(self._h, ctypes.addressof(p), _ptr(d_coords),
                                            _ptr(d_offsets), n, _ptr(d_draws), _ptr(d_count)),
                    "vox_draw_list")

    def capture_graph(self, d_coords, d_nbr_mask, n: int, d_out0, d_out1, cap_faces: int,
                      d_offsets, chunk_index_base: int = 0) -> "Graph":
        """vox_graph_capture: one fused batch launch captured as a CUDA graph."""
        h = _P()
        self._check(self._lib.vox_graph_capture(self._h, _ptr(d_coords), _ptr(d_nbr_mask), n,
                                                chunk_index_base, _ptr(d_out0), _ptr(d_out1),
                                                cap_faces, _ptr(d_offsets), ctypes.byref(h)),
                    "vox_graph_capture")
        g = Graph(self, h)
        self._graphs.add(g)
        return g

    def frustum_cull(self, planes, d_coords, n: int, d_visible):
        """vox_frustum_cull (Frustum::contains, src/frustum_culling.rs:16-40) per chunk."""
        p = (ctypes.c_float * 24)(*[float(v) for v in planes])
        self._check(self._lib.vox_frustum_cull(self._h, ctypes.addressof(p), _ptr(d_coords), n,
                                               _ptr(d_visible)), "vox_frustum_cull")


class Graph:
    """A captured fused batch launch (vox_graph_*); replays on its context's stream."""

    def __init__(self, ctx: "Context", handle):
        self._ctx = ctx
        self._h = handle

    def launch(self):
        """vox_graph_launch: one replay on the context's stream."""
        self._ctx._check(self._ctx._lib.vox_graph_launch(self._h), "vox_graph_launch")

    def close(self):
        """vox_graph_destroy."""
        if self._h:
            self._ctx._lib.vox_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        # no CUDA calls while the interpreter shuts down: the runtime may be gone already
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def camera_matrix(eye, direction, aspect=16 / 9, fovy=1.0471976, znear=0.1, zfar=1000.0):
    """Camera::update_global_matrix (src/camera.rs:41-51), column-major 16 floats."""
    e = (ctypes.c_float * 3)(*eye)
    d = (ctypes.c_float * 3)(*direction)
    out = (ctypes.c_float * 16)()
    st = lib().vox_camera_global_matrix(ctypes.addressof(e), ctypes.addressof(d), aspect, fovy,
                                        znear, zfar, ctypes.addressof(out))
    if st != VOX_OK:
        raise VoxError(st, "vox_camera_global_matrix")
    return list(out)


class Server:
    """The chunk streaming engine (include/voxgpu_serve.h)."""

    def __init__(self, chunk_cfg: Config, view_radius=24, y_min=0, y_max=0, max_batch=64,
                 slots=3, cache_budget_bytes=24 << 30, neighbour_rebuild=False):
        self._lib = lib()
        self.cfg = ServeConfig(chunk_cfg, view_radius, y_min, y_max, max_batch, slots,
                               cache_budget_bytes, 1 if neighbour_rebuild else 0)
        h = _P()
        st = self._lib.vox_serve_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if st != VOX_OK:
            raise VoxError(st, "vox_serve_create")
        self._h = h

    def close(self):
        """vox_serve_destroy."""
        if getattr(self, "_h", None):
            self._lib.vox_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        # no CUDA calls while the interpreter shuts down: the runtime may be gone already
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def now() -> float:
        """The engine clock (vox_serve_now), in seconds."""
        return lib().vox_serve_now()

    def frame(self, view_proj, eye, now=-1.0):
        """vox_serve_frame: one camera frame (ChunkGenerator::build_chunks + World::update):
        cull the view disk, request the visible chunks, admit batches."""
        m = (ctypes.c_float * 16)(*[float(v) for v in view_proj])
        e = (ctypes.c_float * 3)(*[float(v) for v in eye])
        st = self._lib.vox_serve_frame(self._h, ctypes.addressof(m), ctypes.addressof(e), now)
        if st != VOX_OK:
            raise VoxError(st, "vox_serve_frame")

    def drain(self):
        """vox_serve_drain: waits until every request and rebuild is resident."""
        st = self._lib.vox_serve_drain(self._h)
        if st != VOX_OK:
            raise VoxError(st, "vox_serve_drain")

    def submit(self, coords, now=-1.0):
        """vox_serve_submit: request ids of the chunks (existing ids for known chunks)."""
        import numpy as np
        c = np.ascontiguousarray(np.asarray(coords, np.int32).reshape(-1, 3))
        ids = np.zeros(len(c), np.uint64)
        st = self._lib.vox_serve_submit(self._h, c.ctypes.data, len(c), now, ids.ctypes.data)
        if st != VOX_OK:
            raise VoxError(st, "vox_serve_submit")
        return ids.tolist()

    def poll(self, req_id) -> int:
        """VOX_REQ_UNKNOWN, VOX_REQ_PENDING or VOX_REQ_RESIDENT."""
        state = ctypes.c_int32()
        st = self._lib.vox_serve_poll(self._h, req_id, ctypes.byref(state))
        if st != VOX_OK:
            raise VoxError(st, "vox_serve_poll")
        return state.value

    def wait(self, req_id, timeout_s=10.0) -> int:
        """vox_serve_wait; returns the status (VOX_OK when resident)."""
        return self._lib.vox_serve_wait(self._h, req_id, timeout_s)

    def cancel(self, req_id) -> int:
        """vox_serve_cancel; returns the status (VOX_OK when the request was withdrawn)."""
        return self._lib.vox_serve_cancel(self._h, req_id)

    def stats(self) -> ServeStats:
        """vox_serve_get_stats: counters and p50/p99/max latency over every request."""
        s = ServeStats()
        st = self._lib.vox_serve_get_stats(self._h, ctypes.byref(s))
        if st != VOX_OK:
            raise VoxError(st, "vox_serve_get_stats")
        return s

    def latency(self, requested_after=-1e300):
        """(p50 ms, p99 ms, max ms, count) over requests issued at or after the given
        engine-clock time."""
        p50, p99, mx, cnt = (ctypes.c_double(), ctypes.c_double(), ctypes.c_double(),
                             ctypes.c_uint64())
        st = self._lib.vox_serve_latency(self._h, requested_after, ctypes.byref(p50),
                                         ctypes.byref(p99), ctypes.byref(mx), ctypes.byref(cnt))
        if st != VOX_OK:
            raise VoxError(st, "vox_serve_latency")
        return p50.value, p99.value, mx.value, cnt.value

    def lookup(self, coord):
        """(device ptr out0, device ptr out1, faces) of a resident chunk, or None."""
        p0, p1, f = _P(), _P(), ctypes.c_uint64()
        st = self._lib.vox_serve_lookup(self._h, ChunkCoord(*coord), ctypes.byref(p0),
                                        ctypes.byref(p1), ctypes.byref(f))
        if st != VOX_OK:
            return None
        return int(p0.value or 0), int(p1.value or 0), int(f.value)


def serving_camera(t, speed=20.0, yaw_rate=90.0, height=60.0, pitch_deg=-20.0):
    """The simulated camera of the serving workload at time t (seconds): a straight line
    along +x at `speed` units/s with a yaw sweep of `yaw_rate` degrees/s."""
    import math
    eye = (speed * t, height, 0.0)
    yaw = math.radians(270.0 + yaw_rate * t)  # the reference camera starts at yaw 270
    pitch = math.radians(pitch_deg)
    d = (math.cos(yaw) * math.cos(pitch), math.sin(pitch), math.sin(yaw) * math.cos(pitch))
    return eye, d


def grid_coords(xs, ys, zs):
    """Chunk coordinates of a box, in y-major then z then x order (row-major over y, z, x)."""
    return [(x, y, z) for y in ys for z in zs for x in xs]


def neighbour_masks(coords, full6: bool = False):
    """Bit d set iff the neighbour in direction d (-x, +x, -z, +z, -y, +y) is in `coords`
    (the World.chunks lookup of src/chunk_builder.rs:134-169)."""
    present = set(map(tuple, coords))
    offs = [(-1, 0, 0), (1, 0, 0), (0, 0, -1), (0, 0, 1), (0, -1, 0), (0, 1, 0)]
    out = []
    for (x, y, z) in coords:
        m = 0
        for d, (dx, dy, dz) in enumerate(offs):
            if d >= 4 and not full6:
                continue
            if (x + dx, y + dy, z + dz) in present:
                m |= 1 << d
        out.append(m)
    return out


@dataclass(frozen=True)
class Workload:
    """A named synthetic workload (chunk coordinates + generator config)."""
    name: str
    cfg_kwargs: dict
    coords: tuple
    index_base: int = 0
    isolated: bool = False

    def config(self, layout=LAYOUT_VERTEX, cull_mode=CULL_REFERENCE) -> Config:
        """The workload's vox_config with the given layout and cull mode."""
        kw = dict(self.cfg_kwargs)
        kw.setdefault("layout", layout)
        kw.setdefault("cull_mode", cull_mode)
        return make_config(**kw)

    def masks(self, full6: bool = False):
        """Loaded-neighbour masks of the workload's chunks (all 0 for isolated chunks)."""
        if self.isolated:
            return [0] * len(self.coords)
        return neighbour_masks(self.coords, full6)


def workload(name: str) -> Workload:
    """The synthetic workloads of the benchmark suite.

    plain      8x8 chunks of 32^3 around the origin, 2-D Perlin heightmap (perm seed 42,
               f = 1/64, amplitude 12, base 4)
    heightmap  32x32 chunks of 16^3, 2-D fBm 4 octaves (lacunarity 2, gain 0.5,
               f = 1/128), seed 7, amplitude 48, base 8
    density    16x16x16 chunks of 32^3, 3-D fBm 3 octaves (f = 1/96, lacunarity 2,
               gain 0.5), seed 1234, solid iff fbm - (y - 256)/64 > 0
    stress     2048 isolated chunks of 64^3, Bernoulli(0.5) from splitmix64(99 ^ index)
    """
    if name == "plain":
        return Workload(name, dict(chunk_size=32, kind=GEN_HEIGHTMAP, octaves=1, seed=42,
                                   frequency=1.0 / 64, amplitude=12.0, base_height=4.0),
                        tuple(grid_coords(range(-4, 4), [0], range(-4, 4))))
    if name == "heightmap":
        return Workload(name, dict(chunk_size=16, kind=GEN_HEIGHTMAP, octaves=4, seed=7,
                                   frequency=1.0 / 128, lacunarity=2.0, gain=0.5, amplitude=48.0,
                                   base_height=8.0),
                        tuple(grid_coords(range(-16, 16), [0], range(-16, 16))))
    if name == "density":
        return Workload(name, dict(chunk_size=32, kind=GEN_DENSITY, octaves=3, seed=1234,
                                   frequency=1.0 / 96, lacunarity=2.0, gain=0.5, y_ref=256.0,
                                   y_scale=1.0 / 64),
                        tuple(grid_coords(range(16), range(16), range(16))))
    if name == "stress":
        return Workload(name, dict(chunk_size=64, kind=GEN_BERNOULLI, seed=99),
                        tuple((i, 0, 0) for i in range(2048)), isolated=True)
    raise KeyError(name)
