"""Writes tests/golden/oracle_digests.json: SHA-256 digests of the CPU oracle's outputs on
small, fixed cases of every workload and layout, plus a few values in full.

The reference ships no golden vectors; these fixtures pin the oracle itself (any change
to its arithmetic or emission order shows up as a digest change). Regenerate only on a
deliberate change of the specification:

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "wgpu-voxel-engine_gb300"), os.path.join(REPO, "oracle")]

import numpy as np  # noqa: E402

import voxgpu  # noqa: E402
import vox_oracle  # noqa: E402


def cases():
    """(name, config, coords, masks, index_base) of the pinned cases."""
    out = []
    for layout, lname in ((voxgpu.LAYOUT_VERTEX, "vertex"), (voxgpu.LAYOUT_INSTANCED, "instanced")):
        wl = voxgpu.workload("plain")
        coords = list(wl.coords[:8])
        out.append((f"plain/{lname}", wl.config(layout=layout), coords,
                    voxgpu.neighbour_masks(coords), 0))
        wl = voxgpu.workload("heightmap")
        coords = list(wl.coords[:96])
        out.append((f"heightmap/{lname}", wl.config(layout=layout), coords,
                    voxgpu.neighbour_masks(coords), 0))
        wl = voxgpu.workload("density")
        coords = voxgpu.grid_coords(range(5, 7), range(7, 9), range(5, 7))
        out.append((f"density/{lname}", wl.config(layout=layout), coords,
                    voxgpu.neighbour_masks(coords), 0))
        wl = voxgpu.workload("stress")
        out.append((f"stress/{lname}", wl.config(layout=layout), [(0, 0, 0)], None, 77))
    return out


def digest(cfg, coords, masks, base):
    o0, o1, offs = vox_oracle.gen_mesh_batch(cfg, coords, masks, base)
    occ = [vox_oracle.cubes_to_occ(cfg.chunk_size, vox_oracle.generate_cubes(cfg, c, base + i))
           for i, c in enumerate(coords)]
    return {
        "faces": int(offs[-1]),
        "offsets_sha256": hashlib.sha256(np.asarray(offs, np.uint64).tobytes()).hexdigest(),
        "out0_sha256": hashlib.sha256(o0.tobytes()).hexdigest(),
        "out1_sha256": hashlib.sha256(o1.tobytes()).hexdigest(),
        "occupancy_sha256": hashlib.sha256(np.concatenate(occ).tobytes()).hexdigest(),
        "first_face_out0_hex": o0[:96].tobytes().hex() if len(o0) else "",
    }


# Camera views of the plain workload (Camera::update_global_matrix) for the rasteriser.
RASTER_VIEWS = [((60.0, 45.0, 70.0), (-0.6, -0.45, -0.65)), ((0.5, 20.0, 0.5), (0.3, -0.25, 1.0))]
RASTER_SIZE = (320, 180)


def raster_images():
    """The oracle's renders of the plain workload's mesh from RASTER_VIEWS."""
    wl = voxgpu.workload("plain")
    cfg = wl.config()
    o0, o1, offs = vox_oracle.gen_mesh_batch(cfg, wl.coords, wl.masks())
    W, H = RASTER_SIZE
    return [vox_oracle.raster(voxgpu.camera_matrix(eye, d, zfar=400.0), o0, o1, int(offs[-1]), W, H,
                              cfg.texture_index) for eye, d in RASTER_VIEWS]


def write_png(path, img):
    """A minimal RGB PNG (stored scanlines, zlib) for looking at a render."""
    import struct
    import zlib
    h, w = img.shape[:2]
    raw = b"".join(b"\x00" + img[y, :, :3].tobytes() for y in range(h))

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(raw, 9)) + chunk(b"IEND", b""))


def main():
    data = {name: digest(cfg, coords, masks, base) for name, cfg, coords, masks, base in cases()}
    data["perm42_first16"] = vox_oracle.perm(42)[:16].tolist()
    imgs = raster_images()
    data["raster_plain_sha256"] = [hashlib.sha256(im.tobytes()).hexdigest() for im in imgs]
    for k, im in enumerate(imgs):
        write_png(os.path.join(HERE, f"raster_plain_view{k}.png"), im)
    with open(os.path.join(HERE, "oracle_digests.json"), "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
