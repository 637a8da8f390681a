"""Host-only C++ tests of the façade headers (scene loader, JSON reader),
compiled with g++ and run here; no GPU needed."""
import os
import subprocess

from conftest import ROOT


def _compile_and_run(src, out, extra=()):
    exe = os.path.join(out, os.path.splitext(os.path.basename(src))[0])
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "tests", "cpp"), src, "-o", exe, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_scene_loader_cases(tmp_path):
    out = _compile_and_run(os.path.join(ROOT, "tests", "cpp", "test_scene_loader.cpp"), str(tmp_path))
    assert "0 failure(s)" in out


def test_cpp_facade_compiles(tmp_path):
    """The façade headers (ParticleStore, DeviceBuffer, CellGrid, DFSPHSolver)
    and their GPU unit tests compile and link here; they run in the GPU suite."""
    from water_simulation_gb300 import _build

    lib = _build.build()
    cuda = os.path.dirname(os.path.dirname(_build.nvcc()))
    exe = str(tmp_path / "test_facade")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "tests", "cpp"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_facade.cpp"), "-o", exe, "-L", os.path.dirname(lib),
           "-ldfsph_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
