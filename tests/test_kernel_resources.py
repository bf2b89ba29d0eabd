"""Register budgets of the hot kernels, read from ptxas's resource report (no GPU needed).

Occupancy is part of these kernels' design: the 16^3 heightmap launch runs 4 CTAs of 256
threads per SM (64 registers a thread), the density generator 2 CTAs of 512, the stress
launch 2 CTAs of 512. A change that lets the compiler take more registers halves the
resident warps and shows up only as a slower bench, so the budgets are checked here.
"""
import os
import re
import subprocess

import pytest

from voxgpu import _build

NVCC = os.path.join(_build._cuda_home(), "bin", "nvcc")

pytestmark = pytest.mark.skipif(not os.path.exists(NVCC), reason="nvcc not found")


def compile_units(units, tmp_path):
    """{unit: {kernel (mangled): [registers, spill store bytes]}}, the units compiled in
    parallel."""
    procs = {}
    for unit in units:
        src = os.path.join(_build.CSRC, unit)
        cmd = [NVCC] + _build.ARCH + ["-O3", "-std=c++17", "-fmad=false", "-Xptxas", "-v",
                                      "-I", _build.INCLUDE, "-I", _build.CSRC, "-c", src,
                                      "-o", str(tmp_path / (unit + ".o"))]
        procs[unit] = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    out = {}
    for unit, proc in procs.items():
        _, err = proc.communicate()
        assert proc.returncode == 0, err[-2000:]
        res, name = {}, None
        for line in err.splitlines():
            m = re.search(r"Compiling entry function '(\w+)'", line)
            if m:
                name = m.group(1)
                res[name] = [None, 0]
            m = re.search(r"(\d+) bytes spill stores", line)
            if m and name:
                res[name][1] = int(m.group(1))
            m = re.search(r"Used (\d+) registers", line)
            if m and name:
                res[name][0] = int(m.group(1))
        out[unit] = res
    return out


def find(res, stem, *params):
    """The entry whose mangled name is stem<params...> (template ints in order)."""
    tail = "".join(f"ELi{p}" for p in params[1:])
    key = f"{stem}ILi{params[0]}{tail}E"
    hits = [k for k in res if key in k]
    assert hits, f"{stem}{params} not found"
    return res[hits[0]]


@pytest.fixture(scope="module")
def units(tmp_path_factory):
    return compile_units(["vox_kernels_n16.cu", "vox_kernels_n32.cu", "vox_kernels_n64.cu"],
                         tmp_path_factory.mktemp("ptxas"))


@pytest.fixture(scope="module")
def n16(units):
    return units["vox_kernels_n16.cu"]


@pytest.fixture(scope="module")
def n32(units):
    return units["vox_kernels_n32.cu"]


@pytest.fixture(scope="module")
def n64(units):
    return units["vox_kernels_n64.cu"]


@pytest.mark.parametrize("stem", ["k_mesh_batch_overlap", "k_mesh_batch_phased", "k_mesh_batch"])
@pytest.mark.parametrize("gm", [0, 1])  # from resident occupancy; heightmap generation
@pytest.mark.parametrize("layout", [0, 1])
def test_heightmap_16_meshing_kernels_fit_four_ctas_per_sm(n16, stem, gm, layout):
    regs, spill = find(n16, stem, 16, gm, layout, 256)
    assert regs <= 64, f"{stem}<16,{gm},{layout},256>: {regs} registers"


def test_density_32_generation_fits_two_ctas_per_sm(n32):
    regs, spill = find(n32, "k_generate", 32, 2, 512)
    assert regs <= 64
    assert spill <= 64  # a few bytes outside the sample loop


@pytest.mark.parametrize("stem", ["k_mesh_batch_overlap", "k_mesh_batch_phased"])
def test_density_32_fused_kernels_keep_their_budget(n32, stem):
    assert find(n32, stem, 32, 2, 0, 256)[0] <= 80   # 3 CTAs of 256
    assert find(n32, stem, 32, 2, 0, 512)[0] <= 64   # 2 CTAs of 512


def test_heightmap_generation_budget(n16):
    assert find(n16, "k_generate", 16, 1, 256)[0] <= 32


@pytest.mark.parametrize("stem", ["k_mesh_batch_overlap", "k_mesh_batch_phased"])
@pytest.mark.parametrize("layout", [0, 1])
def test_stress_64_kernels_fit_two_ctas_of_512(n64, stem, layout):
    assert find(n64, stem, 64, 3, layout, 512)[0] <= 64
