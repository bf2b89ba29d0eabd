"""The streaming engine's bookkeeping maps (host/vox_flat_map.h) against std::unordered_map,
by a randomized C++ check compiled here (CPU only)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not found")
def test_flat_map_matches_unordered_map(tmp_path):
    exe = str(tmp_path / "flat_map_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall",
                    "-I", os.path.join(REPO, "include"),
                    "-I", os.path.join(REPO, "wgpu-voxel-engine_gb300", "host"),
                    os.path.join(HERE, "flat_map_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
