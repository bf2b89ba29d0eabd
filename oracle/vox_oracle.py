"""ctypes wrapper of the CPU oracle (liboracle_vox.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline legs, to compare the CUDA path's outputs with. Parity status: unpinned (see
vox_oracle.h).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_vox.so")

_LIB = None
_P = ctypes.c_void_p


class _Coord(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int32), ("y", ctypes.c_int32), ("z", ctypes.c_int32)]


def load() -> ctypes.CDLL:
    """Loads liboracle_vox.so (built on first use) and declares its functions."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        import sys
        sys.path.insert(0, os.path.join(os.path.dirname(HERE), "wgpu-voxel-engine_gb300"))
        from voxgpu import _build  # noqa: E402
        _build.build_oracle()
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "or_splitmix64_next": (ctypes.c_uint64, [ctypes.POINTER(ctypes.c_uint64)]),
        "or_perm_init": (None, [ctypes.c_uint64, _P]),
        "or_noise2_f32": (ctypes.c_float, [_P, ctypes.c_float, ctypes.c_float]),
        "or_noise3_f32": (ctypes.c_float, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
        "or_noise2_f64": (ctypes.c_double, [_P, ctypes.c_double, ctypes.c_double]),
        "or_noise3_f64": (ctypes.c_double, [_P, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double]),
        "or_generate_cubes": (ctypes.c_int, [_P, _Coord, ctypes.c_int64, _P]),
        "or_cubes_to_occ": (None, [ctypes.c_int, _P, _P]),
        "or_occ_to_cubes": (None, [ctypes.c_int, _P, _P]),
        "or_cull_faces": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int, _P, _P, _P,
                                           ctypes.c_int64]),
        "or_face_rotation": (None, [ctypes.c_int, _P]),
        "or_instance_raw": (None, [ctypes.c_int, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                   ctypes.c_uint32, _P]),
        "or_face_vertices": (None, [ctypes.c_int, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_uint32, _P, _P]),
        "or_dir_slot": (ctypes.c_int, [ctypes.c_int]),
        "or_mesh_chunk": (ctypes.c_int64, [_P, _Coord, _P, _P, _P, _P, ctypes.c_int64]),
        "or_gen_mesh_batch": (ctypes.c_int64, [_P, _P, _P, ctypes.c_int32, ctypes.c_int64, _P, _P,
                                               ctypes.c_int64, _P]),
        "or_baseline_run": (ctypes.c_int64, [_P, _P, _P, ctypes.c_int32, ctypes.c_int64,
                                             ctypes.c_int]),
        "or_frustum_planes": (None, [_P, _P]),
        "or_frustum_contains": (ctypes.c_int, [_P, _Coord, ctypes.c_int]),
        "or_raster": (None, [_P, _P, _P, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, _P, _P]),
        "or_digest": (ctypes.c_uint64, [_P, ctypes.c_uint64]),
        "or_chunk_digests": (None, [_P, _P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_int, _P]),
        "or_gen_mesh_digests": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int64,
                                               ctypes.c_int, _P, _P]),
        "or_camera_global_matrix": (ctypes.c_int, [_P, _P, ctypes.c_float, ctypes.c_float,
                                                   ctypes.c_float, ctypes.c_float, _P]),
        "or_noise_error_stats": (ctypes.c_int, [_P, _P, ctypes.c_int32,
                                                ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_int64),
                                                ctypes.POINTER(ctypes.c_int64)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def _addr(a) -> int:
    return 0 if a is None else int(a.ctypes.data)


def _cfg_addr(cfg) -> int:
    return ctypes.addressof(cfg)


def coords_array(coords) -> np.ndarray:
    """Chunk coordinates as a contiguous (n, 3) int32 array."""
    return np.ascontiguousarray(np.asarray(coords, dtype=np.int32).reshape(-1, 3))


def perm(seed: int) -> np.ndarray:
    """The doubled noise permutation (512 bytes): Fisher-Yates over splitmix64(seed)."""
    p = np.zeros(512, np.uint8)
    load().or_perm_init(seed, _addr(p))
    return p


def generate_cubes(cfg, coord, chunk_index: int = 0) -> np.ndarray:
    """Chunk::new / generate_terrain (src/chunk.rs:21-46): the chunk's cubes, one byte per
    voxel at x + N z + N^2 y (GRASS 0, AIR 2)."""
    n = cfg.chunk_size
    out = np.zeros(n * n * n, np.uint8)
    st = load().or_generate_cubes(_cfg_addr(cfg), _Coord(*coord), chunk_index, _addr(out))
    assert st == 0, st
    return out


def cubes_to_occ(n: int, cubes: np.ndarray) -> np.ndarray:
    """Cubes to occupancy rows (bit x of row y * N + z; a voxel is solid iff not AIR)."""
    w = n // 32 if n > 32 else 1
    occ = np.zeros(n * n * w, np.uint32)
    load().or_cubes_to_occ(n, _addr(np.ascontiguousarray(cubes, np.uint8)), _addr(occ))
    return occ


def occ_to_cubes(n: int, occ: np.ndarray) -> np.ndarray:
    """Occupancy rows back to cubes."""
    cubes = np.zeros(n * n * n, np.uint8)
    load().or_occ_to_cubes(n, _addr(np.ascontiguousarray(occ, np.uint32)), _addr(cubes))
    return cubes


def _adj_array(adj):
    adj = list(adj or []) + [None] * 6
    keep = [None if a is None else np.ascontiguousarray(a, np.uint8) for a in adj[:6]]
    arr = (_P * 6)(*[_P(_addr(a)) for a in keep])
    return arr, keep


def cull_faces(n: int, cull_mode: int, cubes: np.ndarray, adj=None) -> np.ndarray:
    """Faces as an (F, 4) uint8 array of (x, y, z, dir) in emission order."""
    arr, keep = _adj_array(adj)
    cubes = np.ascontiguousarray(cubes, np.uint8)
    L = load()
    cnt = L.or_cull_faces(n, cull_mode, _addr(cubes), ctypes.addressof(arr), None, 0)
    out = np.zeros((max(cnt, 1), 4), np.uint8)
    L.or_cull_faces(n, cull_mode, _addr(cubes), ctypes.addressof(arr), _addr(out), cnt)
    del keep
    return out[:cnt]


def face_rotation(d: int) -> np.ndarray:
    """The 3x3 f32 rotation of face direction d (src/quad.rs:14-54: Rz * Ry * Rx)."""
    r = np.zeros((3, 3), np.float32)
    load().or_face_rotation(d, _addr(r))
    return r


def bytes_per_face(layout: int):
    """(out0, out1) bytes per face: instanced (68, 0), vertex/index (96, 24)."""
    return (68, 0) if layout == 1 else (96, 24)


def mesh_chunk(cfg, coord, cubes, adj=None):
    """Returns (out0 bytes, out1 bytes, face count) of one chunk."""
    arr, keep = _adj_array(adj)
    cubes = np.ascontiguousarray(cubes, np.uint8)
    L = load()
    cnt = L.or_mesh_chunk(_cfg_addr(cfg), _Coord(*coord), _addr(cubes), ctypes.addressof(arr),
                          None, None, 0)
    b0, b1 = bytes_per_face(cfg.layout)
    o0 = np.zeros(max(cnt, 1) * b0, np.uint8)
    o1 = np.zeros(max(cnt, 1) * max(b1, 1), np.uint8)
    L.or_mesh_chunk(_cfg_addr(cfg), _Coord(*coord), _addr(cubes), ctypes.addressof(arr),
                    _addr(o0), _addr(o1), cnt)
    del keep
    return o0[:cnt * b0], o1[:cnt * b1], cnt


def gen_mesh_batch(cfg, coords, masks=None, index_base: int = 0, cap: int | None = None):
    """Oracle of vox_gen_mesh_batch: (out0 bytes, out1 bytes, offsets[n+1])."""
    c = coords_array(coords)
    n = len(c)
    m = None if masks is None else np.ascontiguousarray(np.asarray(masks, np.uint8))
    L = load()
    offs = np.zeros(n + 1, np.uint64)
    total = L.or_gen_mesh_batch(_cfg_addr(cfg), _addr(c), _addr(m), n, index_base, None, None, 0,
                                _addr(offs))
    if cap is None:
        cap = total
    b0, b1 = bytes_per_face(cfg.layout)
    o0 = np.zeros(max(cap, 1) * b0, np.uint8)
    o1 = np.zeros(max(cap, 1) * max(b1, 1), np.uint8)
    L.or_gen_mesh_batch(_cfg_addr(cfg), _addr(c), _addr(m), n, index_base, _addr(o0), _addr(o1),
                        cap, _addr(offs))
    w = min(total, cap)
    return o0[:w * b0], o1[:w * b1], offs


def baseline_run(cfg, coords, masks, index_base: int, nthreads: int) -> int:
    """The reference's pool work on the CPU: Chunk::new then create_mesh for every chunk,
    one chunk per task on nthreads threads (src/chunk_builder.rs:80-84); returns the faces."""
    c = coords_array(coords)
    m = None if masks is None else np.ascontiguousarray(np.asarray(masks, np.uint8))
    return int(load().or_baseline_run(_cfg_addr(cfg), _addr(c), _addr(m), len(c), index_base,
                                      nthreads))


def _threads(nthreads):
    return nthreads or os.cpu_count() or 1


def digest(data) -> int:
    """or_digest of a byte buffer (numpy array or bytes)."""
    a = np.ascontiguousarray(np.frombuffer(data, np.uint8) if isinstance(data, (bytes, bytearray))
                             else np.asarray(data).view(np.uint8).reshape(-1))
    return int(load().or_digest(_addr(a), a.nbytes))


def chunk_digests(out0, out1, offsets, b0: int, b1: int, nthreads: int = 0) -> np.ndarray:
    """Per-chunk (out0, out1) digests of a meshed batch held in host memory: (n, 2) uint64."""
    offs = np.ascontiguousarray(np.asarray(offsets, np.uint64))
    n = len(offs) - 1
    o0 = np.ascontiguousarray(out0).view(np.uint8).reshape(-1)
    o1 = None if b1 == 0 else np.ascontiguousarray(out1).view(np.uint8).reshape(-1)
    assert o0.nbytes >= int(offs[-1]) * b0 and (o1 is None or o1.nbytes >= int(offs[-1]) * b1)
    out = np.zeros((n, 2), np.uint64)
    load().or_chunk_digests(_addr(o0), _addr(o1), _addr(offs), n, b0, b1, _threads(nthreads),
                            _addr(out))
    return out


def gen_mesh_digests(cfg, coords, masks=None, index_base: int = 0, nthreads: int = 0,
                     counts_only: bool = False):
    """Per-chunk face counts and (out0, out1) digests of or_gen_mesh_batch's output, chunk
    by chunk on nthreads threads (all host threads by default): (counts[n], digests[n, 2])."""
    c = coords_array(coords)
    n = len(c)
    m = None if masks is None else np.ascontiguousarray(np.asarray(masks, np.uint8))
    counts = np.zeros(n, np.uint64)
    dig = None if counts_only else np.zeros((n, 2), np.uint64)
    st = load().or_gen_mesh_digests(_cfg_addr(cfg), _addr(c), _addr(m), n, index_base,
                                    _threads(nthreads), _addr(counts), _addr(dig))
    assert st == 0, st
    return counts, dig


def camera_global_matrix(eye, direction, aspect, fovy, znear, zfar) -> np.ndarray:
    """Camera::update_global_matrix (src/camera.rs:41-51), column-major float32[16]."""
    e = np.ascontiguousarray(np.asarray(eye, np.float32).reshape(3))
    d = np.ascontiguousarray(np.asarray(direction, np.float32).reshape(3))
    out = np.zeros(16, np.float32)
    st = load().or_camera_global_matrix(_addr(e), _addr(d), aspect, fovy, znear, zfar, _addr(out))
    assert st == 0, st
    return out


def frustum_planes(m_colmajor) -> np.ndarray:
    """Frustum::matrix_to_planes (src/frustum_culling.rs:47-85): six planes (a, b, c, d)."""
    m = np.ascontiguousarray(np.asarray(m_colmajor, np.float32).reshape(16))
    out = np.zeros(24, np.float32)
    load().or_frustum_planes(_addr(m), _addr(out))
    return out


def frustum_contains(planes, coord, extent: int) -> bool:
    """Frustum::contains (src/frustum_culling.rs:16-40) for the chunk at coord."""
    p = np.ascontiguousarray(np.asarray(planes, np.float32).reshape(24))
    return bool(load().or_frustum_contains(_addr(p), _Coord(*coord), extent))


def raster(view_proj, vertices, indices, faces: int, width: int, height: int, tex) -> np.ndarray:
    """or_raster: RGBA8 image (height, width, 4) of vertex-layout faces."""
    m = np.ascontiguousarray(np.asarray(view_proj, np.float32).reshape(16))
    v = np.ascontiguousarray(np.frombuffer(bytes(vertices), np.uint8))
    i = np.ascontiguousarray(np.frombuffer(bytes(indices), np.uint8))
    t = np.ascontiguousarray(np.asarray(tex, np.uint32).reshape(6))
    out = np.zeros((height, width, 4), np.uint8)
    load().or_raster(_addr(m), _addr(v), _addr(i), faces, width, height, _addr(t), _addr(out))
    return out


def noise_error_stats(cfg, coords):
    """FP32 against FP64 noise over every voxel of the chunks: (max abs error, voxels within
    that error of the solid threshold, voxels whose solid bit differs)."""
    c = coords_array(coords)
    err = ctypes.c_double()
    near = ctypes.c_int64()
    mism = ctypes.c_int64()
    st = load().or_noise_error_stats(_cfg_addr(cfg), _addr(c), len(c), ctypes.byref(err),
                                     ctypes.byref(near), ctypes.byref(mism))
    assert st == 0, st
    return err.value, near.value, mism.value
