"""The C ABI without a GPU: the library builds, loads and exports every entry point that
include/voxgpu.h declares; argument validation that needs no device works; and calls
that do need a device fail loudly instead of falling back to the CPU."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(REPO, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w \*]*?\b(vox_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("vox_ctx_create", "vox_generate", "vox_mesh", "vox_mesh_batch",
                     "vox_gen_mesh_batch", "vox_gen_mesh_host", "vox_frustum_cull"):
        assert required in names


RUST_BINDING = os.path.join(REPO, "rust", "src", "voxgpu_sys.rs")


def test_rust_binding_covers_every_entry_point():
    """rust/src/voxgpu_sys.rs declares every function of include/*.h, and nothing else."""
    text = open(RUST_BINDING).read()
    bound = set(re.findall(r"pub fn (vox_\w+)\s*\(", text))
    declared = declared_functions()
    missing = [n for n in declared if n not in bound]
    assert not missing, missing
    assert not (bound - set(declared)), sorted(bound - set(declared))


def c_struct_fields():
    """Field names, in order, of every typedef struct of include/*.h."""
    out = {}
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        if not h.endswith(".h"):
            continue
        text = re.sub(r"/\*.*?\*/", "", open(os.path.join(REPO, "include", h)).read(), flags=re.S)
        for body, name in re.findall(r"typedef struct \w+ \{(.*?)\} (\w+);", text, flags=re.S):
            fields = []
            for decl in body.split(";"):
                decl = decl.strip()
                if not decl:
                    continue
                for part in decl.split(","):
                    m = re.search(r"(\w+)\s*(\[[^\]]*\])*\s*$", part.strip())
                    fields.append(m.group(1))
            out[name] = fields
    return out


def test_rust_binding_struct_fields_match_the_headers():
    text = open(RUST_BINDING).read()
    rust = {name: re.findall(r"pub (\w+)\s*:", body)
            for name, body in re.findall(r"pub struct (vox_\w+) \{(.*?)\}", text, flags=re.S)}
    c = c_struct_fields()
    assert c, "no structs parsed from the headers"
    for name, fields in c.items():
        assert name in rust, name
        assert rust[name] == fields, (name, rust[name], fields)


def test_library_exports_every_declared_symbol(vox):
    lib = vox.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_sizes(vox):
    assert vox.lib().vox_abi_version() == 1
    cfg = vox.make_config(chunk_size=32)
    s = vox.query_sizes(cfg)
    assert s.occ_words_per_chunk == 32 * 32
    assert (s.bytes_per_face_out0, s.bytes_per_face_out1) == (96, 24)
    cfg = vox.make_config(chunk_size=64, layout=vox.LAYOUT_INSTANCED)
    s = vox.query_sizes(cfg)
    assert s.occ_words_per_chunk == 64 * 64 * 2
    assert (s.bytes_per_face_out0, s.bytes_per_face_out1) == (68, 0)
    # C layout of vox_config: 3 ints, 6 u32, pad to 8, then vox_generator (48 bytes).
    assert ctypes.sizeof(vox.Generator) == 48
    assert vox.Config.gen.offset == 40 and ctypes.sizeof(vox.Config) == 88
    assert ctypes.sizeof(vox.ChunkCoord) == 12


@pytest.mark.parametrize("field,value", [("chunk_size", 12), ("chunk_size", 128),
                                         ("layout", 7), ("cull_mode", 3)])
def test_invalid_config_rejected(vox, field, value):
    cfg = vox.make_config()
    setattr(cfg, field, value)
    s = vox.Sizes()
    assert vox.lib().vox_query_sizes(ctypes.byref(cfg), ctypes.byref(s)) == vox.VOX_ERR_INVALID


def test_frustum_planes_host_function(vox, oracle):
    import numpy as np
    rng = np.random.default_rng(5)
    m = rng.standard_normal(16).astype(np.float32)
    assert np.array_equal(np.array(vox.frustum_planes(m), np.float32), oracle.frustum_planes(m))


def test_no_cpu_fallback_without_gpu(vox):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible; covered by the gpu tests")
    with pytest.raises(vox.VoxError) as e:
        vox.Context(vox.make_config())
    assert e.value.status in (vox.VOX_ERR_NO_DEVICE, vox.VOX_ERR_CUDA)


def test_struct_layouts_match_the_c_headers(vox, tmp_path):
    """sizeof / offsetof from the C compiler (the public headers) against the ctypes mirrors
    and the documented record sizes."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text("""
#include <stddef.h>
#include <stdio.h>
#include "voxgpu.h"
#include "voxgpu_serve.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n",
         sizeof(vox_chunk_coord), sizeof(vox_generator), sizeof(vox_config),
         offsetof(vox_config, gen), sizeof(vox_vertex), sizeof(vox_instance_raw),
         sizeof(vox_sizes), sizeof(vox_tuning), sizeof(vox_draw_indexed_indirect),
         sizeof(vox_serve_config), sizeof(vox_serve_stats), offsetof(vox_serve_config, view_radius));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [ctypes.sizeof(vox.ChunkCoord), ctypes.sizeof(vox.Generator), ctypes.sizeof(vox.Config),
            vox.Config.gen.offset, 24, 68, ctypes.sizeof(vox.Sizes), ctypes.sizeof(vox.Tuning), 20,
            ctypes.sizeof(vox.ServeConfig), ctypes.sizeof(vox.ServeStats),
            vox.ServeConfig.view_radius.offset]
    assert got == want
