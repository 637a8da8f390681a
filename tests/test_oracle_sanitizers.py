"""The CPU oracle under AddressSanitizer and UndefinedBehaviorSanitizer (the
host half of the sanitizer plan: the GPU side is checked by bit-exact and
element-wise comparisons against this oracle)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_oracle_is_clean_under_asan_and_ubsan(tmp_path):
    exe = tmp_path / "oracle_sanitize"
    src = os.path.join(ROOT, "tests", "cpp", "oracle_sanitize_main.cpp")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-ffp-contract=off",
           "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", src, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("sanitizer runtime unavailable: " + r.stderr[-200:])
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "oracle sanitizer run ok" in r.stdout
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr
