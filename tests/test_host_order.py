"""The streaming engine's admit order (host/vox_order.h: a stable radix sort on squared
distances) against std::stable_sort, by a randomized C++ check compiled here (CPU only)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not found")
def test_radix_order_matches_stable_sort(tmp_path):
    exe = str(tmp_path / "order_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall",
                    "-I", os.path.join(REPO, "wgpu-voxel-engine_gb300", "host"),
                    os.path.join(HERE, "order_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
