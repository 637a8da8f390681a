"""The C++ façade and sim_cli on a GPU: the reference's ParticleStore, CellGrid,
boundary-sampler and DFSPHSolver unit tests written against include/water,
compiled here and run; sim_cli on a small scene with frame recording."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_cpp_facade_unit_tests(tmp_path):
    from water_simulation_gb300 import _build

    lib = _build.build()
    cuda = os.path.dirname(os.path.dirname(_build.nvcc()))
    exe = str(tmp_path / "test_facade")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "tests", "cpp"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_facade.cpp"), "-o", exe, "-L", os.path.dirname(lib),
           "-ldfsph_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr


def test_sim_cli_records_frames(tmp_path):
    from water_simulation_gb300 import _build

    exe = _build.build_sim_cli()
    scene = tmp_path / "drop.json"
    scene.write_text("""{"schema_version": "1.0", "name": "small_drop",
      "output": {"fps": 30, "frame_range": [0, 3], "format": "bin"},
      "scene": {"fluid": {"solver": "dfsph", "particle_radius": 0.01, "rest_density": 1000.0,
                          "viscosity": 0.001, "gravity": [0.0, -9.81, 0.0],
                          "initial_block_min": [0.42, 0.30, 0.42], "initial_block_max": [0.58, 0.44, 0.58]}}}""")
    out = tmp_path / "frames"
    r = subprocess.run([exe, "--scene", str(scene), "--record", "--out", str(out), "--no-vulkan"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "=== sim_cli OK ===" in r.stdout
    frames = sorted(os.listdir(out))
    assert frames == ["frame_0000.bin", "frame_0001.bin", "frame_0002.bin", "frame_0003.bin"]
    raw0 = (out / "frame_0000.bin").read_bytes()
    raw3 = (out / "frame_0003.bin").read_bytes()
    n = struct.unpack("<I", raw0[:4])[0]
    assert n == 9 * 7 * 9 and len(raw3) == 4 + 12 * n
    p0 = np.frombuffer(raw0[4:], np.float32).reshape(n, 3)
    p3 = np.frombuffer(raw3[4:], np.float32).reshape(n, 3)
    assert p3[:, 1].mean() < p0[:, 1].mean()  # it fell
    assert np.isfinite(p3).all()
    bad = subprocess.run([exe, "--scene", str(tmp_path / "missing.json")], capture_output=True, text=True)
    assert bad.returncode == 1 and "cannot open" in bad.stderr


def test_sim_cli_resumes_from_a_state_file(tmp_path):
    # frames 0..3 in one run equal frames 0..2, a state file, then 2..3 resumed
    from water_simulation_gb300 import _build

    exe = _build.build_sim_cli()
    scene = tmp_path / "drop.json"
    scene.write_text("""{"schema_version": "1.0", "name": "small_drop",
      "output": {"fps": 30, "frame_range": [0, 3], "format": "bin"},
      "scene": {"fluid": {"solver": "dfsph", "particle_radius": 0.01, "rest_density": 1000.0,
                          "viscosity": 0.001, "gravity": [0.0, -9.81, 0.0],
                          "initial_block_min": [0.42, 0.30, 0.42], "initial_block_max": [0.58, 0.44, 0.58]}}}""")

    def run(*extra):
        r = subprocess.run([exe, "--scene", str(scene), "--no-vulkan", *extra], capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        return r.stdout

    run("--frames", "0:3", "--record", "--out", str(tmp_path / "a"))
    run("--frames", "0:2", "--save-state", str(tmp_path / "s.bin"))
    out = run("--frames", "2:3", "--load-state", str(tmp_path / "s.bin"), "--record", "--out", str(tmp_path / "b"))
    assert "resumed:" in out
    assert (tmp_path / "a" / "frame_0003.bin").read_bytes() == (tmp_path / "b" / "frame_0003.bin").read_bytes()


def test_sim_cli_applies_solver_params_on_request(tmp_path):
    from water_simulation_gb300 import _build

    exe = _build.build_sim_cli()
    scene = tmp_path / "sp.json"
    scene.write_text("""{"schema_version": "1.0", "name": "sp",
      "output": {"fps": 30, "frame_range": [0, 1], "format": "bin"},
      "scene": {"fluid": {"solver": "dfsph", "particle_radius": 0.01,
                          "initial_block_min": [0.42, 0.30, 0.42], "initial_block_max": [0.58, 0.44, 0.58],
                          "solver_params": {"max_density_iters": 20, "max_divergence_iters": 5,
                                            "eta_density": 1e-4, "eta_divergence": 1e-3, "cfl_lambda": 0.3}}}}""")
    r = subprocess.run([exe, "--scene", str(scene), "--no-vulkan", "--solver-params"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "solver_params: density 20 iters" in r.stdout and "cfl 0.30" in r.stdout
    r = subprocess.run([exe, "--scene", str(scene), "--no-vulkan"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "solver_params:" not in r.stdout  # ignored by default, as the reference does
