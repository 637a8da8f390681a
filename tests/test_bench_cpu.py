"""bench.py's contract on the CPU: the defaults (one GPU, at least 3 warm-up
steps), the per-kernel algorithmic byte counts, and the reference arm's JSON
line (it times the FP32 restatement, so it runs here on a small workload)."""
import argparse
import sys

import bench


def test_defaults_run_one_gpu_with_warmup(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.gpus == 1 and a.impl == "ours" and a.workload == "dam1m"
    assert a.warmup >= 3 and a.steps >= 1


def test_algorithmic_bytes_per_launch():
    n, nb, cells = 1_024_000, 19_602, 8_000_412
    assert bench.algorithmic_bytes("pressure_rate", n, nb, cells) == 40 * n + 16 * nb
    assert bench.algorithmic_bytes("pressure_apply", n, nb, cells) == 44 * n + 16 * nb
    assert bench.algorithmic_bytes("density_alpha", n, nb, cells) == 20 * n + 16 * nb
    assert bench.algorithmic_bytes("grid_scan", n, nb, cells) == 8 * (cells + 1)
    assert bench.algorithmic_bytes("no_such_class", n, nb, cells) is None


def test_reference_arm_line_has_the_contract_keys():
    args = argparse.Namespace(workload="puddle", steps=2, warmup=3, gpus=1, impl="reference")
    line = bench.reference_arm(args, rank=0, world=1)
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["warmup"] == 3
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and "sample" in cb
    e = line["e2e"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0 and e["value"] == line["value"]
    assert line["config"]["workload"] == "puddle_4913"
    # other ranks print nothing and do no work
    assert bench.reference_arm(args, rank=1, world=2) is None


def test_reference_arm_never_loads_the_library():
    """The reference arm times the oracle alone: its scene (walls sampled by
    the oracle) and its configuration are built without libdfsph_gb300.so,
    which must not even be mapped into the process."""
    import os
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import argparse, json, bench\n"
            "a = argparse.Namespace(workload='puddle', steps=1, warmup=3, gpus=1, impl='reference')\n"
            "line = bench.reference_arm(a, rank=0, world=1)\n"
            "maps = open('/proc/self/maps').read()\n"
            "print(json.dumps({'lib': 'libdfsph_gb300' in maps, 'oracle': 'liboracle' in maps,\n"
            "                  'value': line['value'], 'nb': line['config']['boundary_particles']}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    import json

    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["oracle"] and not out["lib"]
    assert out["value"] > 0 and out["nb"] == 46818


def test_reference_arm_scene_is_the_benchmark_scene():
    """The oracle's wall sampler gives the library's walls bit for bit, so the
    arm steps the same input as the library's arm."""
    import numpy as np

    from oracle import oracle as O

    a = bench.make_scene("puddle")
    b = bench.make_scene("puddle", sampler=O.sample_aabb_boundary)
    assert np.array_equal(a.boundary, b.boundary) and np.array_equal(a.fluid, b.fluid)
    c = bench.oracle_config(b)
    d = O.config_from(a.config())
    for name, _ in O.OracleConfig._fields_:
        x, y = getattr(c, name), getattr(d, name)
        assert (list(x) == list(y)) if hasattr(x, "__len__") else x == y, name


def test_both_arms_carry_the_same_config():
    """The reference arm's `config` equals the one the GPU arm prints for the
    same workload (the driver compares them)."""
    from oracle import oracle as O

    args = argparse.Namespace(workload="puddle", steps=1, warmup=3, gpus=1, impl="reference")
    line = bench.reference_arm(args, rank=0, world=1)
    assert line["config"] == bench.workload_config(bench.make_scene("puddle"), 1)
    big = bench.workload_config(bench.make_scene("dam1m", sampler=O.sample_aabb_boundary), 1)
    assert big["particles"] == 1024000 and "touches more" in big["l2"]
