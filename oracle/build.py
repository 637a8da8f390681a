"""Build recipes of the oracle (test infrastructure only).

* liboracle.so      - the C++/OpenMP restatement in dfsph_oracle.cpp (g++).
* _ref/*.fatbin     - the reference's own kernels, compiled from the reference
                      sources where they lie (solvers/dfsph/src/dfsph_kernels.cu,
                      core/src/cell_grid.cu, core/src/spatial_accel.cu) with
                      the reference's flags (-use_fast_math,
                      CMakeLists.txt:56) for sm_103a. Only
                      possible where the reference tree exists; the fatbins are
                      device code, so they run on Arm GPU hosts unchanged.
* _ref/libref_runner.so - ref_runner.cu: host orchestration restating
                      DFSPHSolver / CellGrid::build / SpatialAccel::build
                      around those fatbins (nvcc,
                      built wherever it runs).
Nothing from the reference is copied into this repository; _ref/ is ignored.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
RUNNER_LIB = os.path.join(REF_OUT, "libref_runner.so")
FATBINS = {
    "dfsph_kernels.fatbin": ("solvers/dfsph/src/dfsph_kernels.cu", ["core/include", "solvers/dfsph/include"]),
    "cell_grid.fatbin": ("core/src/cell_grid.cu", ["core/include"]),
    "spatial_accel.fatbin": ("core/src/spatial_accel.cu", ["core/include"]),
}
REFERENCE_ROOT = os.environ.get("WATER_REFERENCE_ROOT", "/root/reference")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target, deps):
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target) for d in deps)


def nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build_oracle(force=False):
    src = os.path.join(HERE, "dfsph_oracle.cpp")
    if force or _stale(ORACLE_LIB, [src]):
        tmp = ORACLE_LIB + ".tmp"
        _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              src, "-o", tmp])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference_fatbins(force=False):
    """Compile the reference kernels; a no-op where the reference tree is absent."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "solvers")):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    for out, (src, incs) in FATBINS.items():
        target = os.path.join(REF_OUT, out)
        srcp = os.path.join(REFERENCE_ROOT, src)
        if force or _stale(target, [srcp]):
            cmd = [nvcc(), "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++20",
                   "--expt-extended-lambda", "--expt-relaxed-constexpr", "-use_fast_math"]
            for i in incs:
                cmd += ["-I", os.path.join(REFERENCE_ROOT, i)]
            _run(cmd + [srcp, "-o", target])
    return True


def have_reference_fatbins():
    return all(os.path.exists(os.path.join(REF_OUT, f)) for f in FATBINS)


def build_runner(force=False):
    """Host runner around the reference fatbins (needs nvcc; links libcuda)."""
    src = os.path.join(HERE, "ref_runner.cu")
    if not os.path.exists(src):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    if force or _stale(RUNNER_LIB, [src]):
        tmp = RUNNER_LIB + ".tmp"
        _run([nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared",
              "-Xcompiler", "-fPIC", src, "-o", tmp, "-lcuda"])
        os.replace(tmp, RUNNER_LIB)
    return RUNNER_LIB


def build_all(force=False):
    build_oracle(force)
    build_reference_fatbins(force)
    if have_reference_fatbins():
        build_runner(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("oracle:", ORACLE_LIB, "fatbins:", have_reference_fatbins())
