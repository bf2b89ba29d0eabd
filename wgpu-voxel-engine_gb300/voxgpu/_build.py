"""In-tree build of the CUDA library (libvoxgpu.so) and of the CPU oracle.

The library is compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``)
with ``-fmad=false`` so that every float expression on the device rounds once per
operation in the written order; host code is compiled with ``-ffp-contract=off`` for
the same reason (GCC contracts a*b+c into an FMA by default on AArch64).

Translation units are compiled in parallel and only when a source or header is newer
than the object, so a rebuild on an unchanged tree takes a fraction of a second.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
SRC_ROOT = os.path.dirname(PKG_DIR)                       # wgpu-voxel-engine_gb300/
REPO = os.path.dirname(SRC_ROOT)
CSRC = os.path.join(SRC_ROOT, "csrc")
HOST = os.path.join(SRC_ROOT, "host")
INCLUDE = os.path.join(REPO, "include")
MACHINE = platform.machine()
BUILD_DIR = os.path.join(SRC_ROOT, "_build", MACHINE)
LIB_PATH = os.path.join(PKG_DIR, "libvoxgpu.so")
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle_vox.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.isdir(cand):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("CUDA toolkit not found (nvcc)")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _stamp_ok(path: str) -> bool:
    """True if `path` exists and was built on this machine architecture."""
    try:
        with open(path + ".arch") as f:
            return os.path.exists(path) and f.read().strip() == MACHINE
    except OSError:
        return False


def _write_stamp(path: str) -> None:
    with open(path + ".arch", "w") as f:
        f.write(MACHINE + "\n")


def _run(cmd):
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout)
    return res.stdout


def build_library(verbose: bool = False, extra_nvcc=None) -> str:
    """Compiles csrc/*.cu and csrc/*.cpp into voxgpu/libvoxgpu.so; returns its path."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    if os.path.isdir(HOST):
        headers += [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    hdr_time = _newest(headers)
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    host = sorted(f for f in os.listdir(HOST) if f.endswith(".cpp")) if os.path.isdir(HOST) else []
    nv_flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                       "-Xcompiler", "-fPIC,-ffp-contract=off",
                       "-I", INCLUDE, "-I", CSRC] + list(extra_nvcc or [])
    cxx = os.environ.get("CXX", "g++")
    cxx_flags = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall",
                 "-I", INCLUDE, "-I", CSRC, "-I", os.path.join(cuda, "include")]
    jobs = []
    objs = []
    for f in cu + cpp + host:
        src = os.path.join(HOST if f in host else CSRC, f)
        obj = os.path.join(BUILD_DIR, f + ".o")
        objs.append(obj)
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
            continue
        if f.endswith(".cu"):
            jobs.append([nvcc] + nv_flags + ["-c", src, "-o", obj])
        else:
            jobs.append([cxx] + cxx_flags + ["-c", src, "-o", obj])
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(workers) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if jobs or not _stamp_ok(LIB_PATH) or os.path.getmtime(LIB_PATH) < _newest(objs):
        tmp = LIB_PATH + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread", "-ldl"])
        os.replace(tmp, LIB_PATH)
        _write_stamp(LIB_PATH)
    return LIB_PATH


def build_oracle() -> str:
    """Compiles the C oracle (test infrastructure) into oracle/liboracle_vox.so."""
    src = os.path.join(ORACLE_DIR, "vox_oracle.c")
    hdrs = [os.path.join(ORACLE_DIR, "vox_oracle.h"), os.path.join(INCLUDE, "voxgpu.h")]
    if _stamp_ok(ORACLE_LIB) and os.path.getmtime(ORACLE_LIB) >= _newest([src] + hdrs):
        return ORACLE_LIB
    cc = os.environ.get("CC", "gcc")
    tmp = ORACLE_LIB + ".tmp"
    _run([cc, "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c11", "-fPIC", "-shared",
          "-Wall", "-o", tmp, src, "-lm", "-lpthread"])
    os.replace(tmp, ORACLE_LIB)
    _write_stamp(ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
    print(build_oracle())
    sys.exit(0)
