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
