"""Build recipe of the native library (libdfsph_gb300.so), in-tree.

nvcc for sm_103a only; every translation unit is compiled in parallel, then
linked into one shared library that exports the C ABI of include/dfsph_gb300.h.
Host code is compiled with -ffp-contract=off so that host float arithmetic (grid
geometry, boundary sampling) is identical on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libdfsph_gb300.so")
# the bounds-checked build (every neighbour run validated, violations counted)
CHECKED_BUILD_DIR = os.path.join(PKG_DIR, "_build_checked")
CHECKED_LIB_PATH = os.path.join(PKG_DIR, "libdfsph_gb300_checked.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-O2",
    "-I", os.path.join(ROOT, "include"),
]
# (source, extra flags)
CUDA_UNITS = [
    ("capi.cu", []),
    ("solver_fp32.cu", []),
    ("solver_fp64.cu", []),
    # the one unit built with the reference's fast math (see its header)
    ("stencil_recip.cu", ["-use_fast_math"]),
    ("static_grid.cu", []),
    ("morton.cu", []),
    ("lbvh.cu", []),
]
CXX_UNITS = ["geometry.cpp"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdfsph_gb300.so")
    return exe


def _sources() -> list[str]:
    out = []
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".cpp", ".h")):
                out.append(os.path.join(d, f))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    """Compile libdfsph_gb300.so (or, checked=True, the bounds-checked
    libdfsph_gb300_checked.so) if any source is newer; returns its path."""
    lib_path = CHECKED_LIB_PATH if checked else LIB_PATH
    build_dir = CHECKED_BUILD_DIR if checked else BUILD_DIR
    deps = _sources()
    if not force and not _stale(lib_path, deps):
        return lib_path
    os.makedirs(build_dir, exist_ok=True)
    nv = nvcc()
    jobs = []
    objs = []
    defs = ["-DDFSPH_BOUNDS_CHECK"] if checked else []
    for src, extra in CUDA_UNITS:
        obj = os.path.join(build_dir, src + ".o")
        objs.append(obj)
        jobs.append([nv] + NVCC_COMMON + defs + extra + ["-c", os.path.join(CSRC, src), "-o", obj])
    for src in CXX_UNITS:
        obj = os.path.join(build_dir, src + ".o")
        objs.append(obj)
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                     "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
                     "-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(_run, jobs))
    tmp = lib_path + ".tmp"
    _run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"])
    os.replace(tmp, lib_path)
    if verbose:
        print("built", lib_path)
    return lib_path


APPS_DIR = os.path.join(PKG_DIR, "apps")
BIN_DIR = os.path.join(PKG_DIR, "bin")
SIM_CLI = os.path.join(BIN_DIR, "sim_cli")


def build_sim_cli(force: bool = False) -> str:
    """The sim_cli driver (host C++ over the C++ façade and libdfsph_gb300.so)."""
    lib = build(force=force)
    src = os.path.join(APPS_DIR, "sim_cli.cpp")
    headers = []
    for d, _, files in os.walk(os.path.join(ROOT, "include")):
        headers += [os.path.join(d, f) for f in files if f.endswith(".h")]
    if not force and not _stale(SIM_CLI, [src, lib] + headers):
        return SIM_CLI
    os.makedirs(BIN_DIR, exist_ok=True)
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    tmp = SIM_CLI + ".tmp"
    _run(["g++", "-std=c++17", "-O2", "-Wall", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
          "-I", os.path.join(cuda, "include"), src, "-o", tmp, "-L", PKG_DIR, "-ldfsph_gb300",
          "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN/.."])
    os.replace(tmp, SIM_CLI)
    return SIM_CLI


if __name__ == "__main__":
    build(force=True, verbose=True)
    build_sim_cli(force=True)
