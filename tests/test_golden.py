"""The CPU oracle against its committed golden digests (tests/golden/make_golden.py), and
the FP32 noise against the FP64 noise (max error and the voxels whose solid bit the FP32
rounding decides)."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_matches_golden_digests(oracle):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden
    want = json.load(open(os.path.join(HERE, "golden", "oracle_digests.json")))
    for name, cfg, coords, masks, base in make_golden.cases():
        assert make_golden.digest(cfg, coords, masks, base) == want[name], name
    assert oracle.perm(42)[:16].tolist() == want["perm42_first16"]


def test_oracle_raster_matches_golden_images(oracle):
    """The oracle's renders of the plain workload (tests/golden/raster_plain_view*.png are
    the same images, for viewing) against their committed digests."""
    import hashlib
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden
    want = json.load(open(os.path.join(HERE, "golden", "oracle_digests.json")))
    got = [hashlib.sha256(im.tobytes()).hexdigest() for im in make_golden.raster_images()]
    assert got == want["raster_plain_sha256"]


@pytest.mark.parametrize("name,max_err,max_mismatch", [("plain", 1e-5, 4), ("heightmap", 5e-5, 4)])
def test_fp32_noise_error_against_fp64(vox, oracle, name, max_err, max_mismatch):
    wl = vox.workload(name)
    err, near, mism = oracle.noise_error_stats(wl.config(), wl.coords)
    assert 0.0 < err < max_err
    assert mism <= max_mismatch
    assert near >= mism  # a flipped voxel lies within the error of the threshold


def test_fp32_density_error_against_fp64(vox, oracle):
    wl = vox.workload("density")
    coords = vox.grid_coords(range(4), range(7, 9), range(4))
    err, near, mism = oracle.noise_error_stats(wl.config(), coords)
    assert 0.0 < err < 1e-5 and mism <= near
