"""The C ABI's error behaviour without a GPU: every entry point called with NULL handles and
NULL or out-of-range arguments returns its documented status (VOX_ERR_INVALID, or VOX_OK
for the destroy calls) before any CUDA work, and never crashes. The reference panics (via
unwrap) where these calls return a status. None of these calls reaches the GPU, so they are
safe on a machine with one too; the calls that would reach it run only without a GPU."""
import ctypes

import pytest

INVALID, OK = 1, 0


def _call(vox, name, *args):
    return getattr(vox.lib(), name)(*args)


# entry point -> (arguments with NULL handles / pointers, expected result)
def _null_cases(vox):
    C = vox.ChunkCoord()
    return {
        "vox_abi_version": ((), None),
        "vox_status_string": ((99,), b"unknown status"),
        "vox_query_sizes": ((None, None), INVALID),
        "vox_ctx_create": ((None, None, None), INVALID),
        "vox_ctx_destroy": ((None,), OK),
        "vox_ctx_sync": ((None,), INVALID),
        "vox_ctx_stream": ((None,), None),
        "vox_ctx_last_error": ((None,), b""),
        "vox_generate": ((None, None, 1, 0, None), INVALID),
        "vox_generate_slots": ((None, None, 1, 0, None, 1, None), INVALID),
        "vox_occ_to_cubes": ((None, None, 1, None), INVALID),
        "vox_cubes_to_occ": ((None, None, 1, None), INVALID),
        "vox_mesh": ((None, None, None, C, None, None, 0, None), INVALID),
        "vox_mesh_batch": ((None, None, 1, None, None, None, 1, None, None, 0, None), INVALID),
        "vox_gen_mesh_batch": ((None, None, None, 1, 0, None, None, 0, None), INVALID),
        "vox_gen_mesh_host": ((None, None, None, 1, 0, None, None, 0, None), INVALID),
        "vox_gen_mesh_batch_noalloc": ((None, None, None, None, 1, 0, None, None, 0, None),
                                       INVALID),
        "vox_frustum_planes": ((None, None), INVALID),
        "vox_frustum_cull": ((None, None, None, 1, None), INVALID),
        "vox_raster": ((None, None, None, None, 0, 8, 8, None, None), INVALID),
        "vox_ctx_get_tuning": ((None, None), INVALID),
        "vox_ctx_set_tuning": ((None, None), INVALID),
        "vox_autotune": ((None, None, None, 1, 0, None, None, 0, None, 1, None), INVALID),
        "vox_selftest_lookback_timeout": ((None, 1), INVALID),
        "vox_graph_capture": ((None, None, None, 1, 0, None, None, 0, None, None), INVALID),
        "vox_graph_launch": ((None,), INVALID),
        "vox_draw_list": ((None, None, None, None, 1, None, None), INVALID),
        "vox_graph_destroy": ((None,), OK),
        "vox_serve_create": ((None, None), INVALID),
        "vox_serve_destroy": ((None,), OK),
        "vox_serve_now": ((), None),
        "vox_serve_frame": ((None, None, None, -1.0), INVALID),
        "vox_serve_drain": ((None,), INVALID),
        "vox_serve_submit": ((None, None, 1, -1.0, None), INVALID),
        "vox_serve_poll": ((None, 1, None), INVALID),
        "vox_serve_wait": ((None, 1, 0.0), INVALID),
        "vox_serve_cancel": ((None, 1), INVALID),
        "vox_serve_get_stats": ((None, None), INVALID),
        "vox_serve_latency": ((None, 0.0, None, None, None, None), INVALID),
        "vox_serve_lookup": ((None, C, None, None, None), INVALID),
        "vox_camera_global_matrix": ((None, None, 1.0, 1.0, 0.1, 10.0, None), INVALID),
        "vox_world_to_chunk": ((None, 16), "zero"),
        "vox_host_alloc": ((16, None), INVALID),
        "vox_host_free": ((None,), OK),
    }


def test_every_entry_point_rejects_null_arguments(vox):
    cases = _null_cases(vox)
    assert set(cases) == set(vox._SIGS), set(vox._SIGS) ^ set(cases)
    for name, (args, want) in cases.items():
        got = _call(vox, name, *args)
        if want == "zero":
            assert (got.x, got.y, got.z) == (0, 0, 0), name
        elif want is not None:
            assert got == want, (name, got, want)


@pytest.mark.parametrize("field,value", [("view_radius", -1), ("max_batch", 0), ("slots", 0),
                                         ("y_max", -1), ("cache_budget_bytes", 0)])
def test_serve_create_rejects_bad_configs(vox, field, value):
    cfg = vox.ServeConfig(vox.make_config(chunk_size=16), 4, 0, 0, 64, 2, 1 << 30, 0)
    setattr(cfg, field, value)
    out = ctypes.c_void_p()
    assert vox.lib().vox_serve_create(ctypes.byref(cfg), ctypes.byref(out)) == INVALID
    assert not out.value


def test_serve_create_rejects_a_bad_chunk_config(vox):
    chunk = vox.make_config()
    chunk.chunk_size = 12
    cfg = vox.ServeConfig(chunk, 4, 0, 0, 64, 2, 1 << 30, 0)
    out = ctypes.c_void_p()
    assert vox.lib().vox_serve_create(ctypes.byref(cfg), ctypes.byref(out)) == INVALID


@pytest.mark.parametrize("octaves", [0, 17])
def test_ctx_create_rejects_octaves_out_of_range(vox, octaves):
    cfg = vox.make_config(octaves=octaves)
    out = ctypes.c_void_p()
    assert vox.lib().vox_ctx_create(ctypes.byref(cfg), None, ctypes.byref(out)) == INVALID
    assert not out.value


def test_noalloc_rejects_bad_counts_before_any_cuda_call(vox):
    cfg = vox.make_config()
    L = vox.lib()
    assert L.vox_gen_mesh_batch_noalloc(ctypes.byref(cfg), None, None, None, -1, 0, None, None,
                                        0, None) == INVALID
    assert L.vox_gen_mesh_batch_noalloc(ctypes.byref(cfg), None, None, None, 16385, 0, None,
                                        None, 0, None) == INVALID
    assert L.vox_gen_mesh_batch_noalloc(ctypes.byref(cfg), None, None, None, 0, 0, None, None,
                                        0, None) == OK


def test_camera_matrix_rejects_degenerate_views(vox):
    L = vox.lib()
    eye = (ctypes.c_float * 3)(0, 0, 0)
    out = (ctypes.c_float * 16)()
    for d, aspect, zn, zf in (((0, 0, 0), 1.0, 0.1, 10.0),   # no direction
                              ((0, 1, 0), 1.0, 0.1, 10.0),   # parallel to up
                              ((1, 0, 0), 0.0, 0.1, 10.0),   # zero aspect
                              ((1, 0, 0), 1.0, 0.0, 10.0),   # znear 0
                              ((1, 0, 0), 1.0, 1.0, 0.5)):   # zfar before znear
        dv = (ctypes.c_float * 3)(*d)
        assert L.vox_camera_global_matrix(eye, dv, aspect, 1.0, zn, zf, out) == INVALID


def test_serve_create_without_a_gpu_fails_cleanly(vox):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible; the engine is covered by the gpu tests")
    cfg = vox.ServeConfig(vox.make_config(chunk_size=16), 4, 0, 0, 64, 2, 1 << 30, 1)
    out = ctypes.c_void_p()
    st = vox.lib().vox_serve_create(ctypes.byref(cfg), ctypes.byref(out))
    assert st in (vox.VOX_ERR_CUDA, vox.VOX_ERR_NO_DEVICE, vox.VOX_ERR_OOM)
    assert not out.value
