"""The resident host-copy pool (csrc/copy_pool.h) on the CPU: three threads
run copy sets of random sizes and functions over numbered pieces at once
through one pool; every byte must arrive, every piece must run once and every
run must return, plain and under ThreadSanitizer."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "heterogeneous-clue_gb300", "csrc")


def _build_and_run(tmp_path, flags, iters, timeout):
    exe = tmp_path / "copy_pool_stress"
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", *flags, "-I" + CSRC, os.path.join(HERE, "copy_pool_stress.cc"),
           "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    p = subprocess.run([str(exe), str(iters)], capture_output=True, text=True, timeout=timeout)
    return p


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_copy_pool_concurrent_sets(tmp_path):
    p = _build_and_run(tmp_path, [], 1000, 120)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "mismatches 0" in p.stdout


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_copy_pool_under_thread_sanitizer(tmp_path):
    try:
        p = _build_and_run(tmp_path, ["-fsanitize=thread", "-g"], 100, 300)
    except subprocess.CalledProcessError as e:  # toolchain without the sanitizer runtime
        pytest.skip("ThreadSanitizer not available: " + e.stderr[-200:])
    if "FATAL: ThreadSanitizer" in p.stderr:  # runtime refuses this kernel's memory layout
        pytest.skip("ThreadSanitizer cannot run here")
    assert p.returncode == 0, p.stdout + p.stderr[-2000:]
    assert "WARNING: ThreadSanitizer" not in p.stderr, p.stderr[-2000:]
    assert "mismatches 0" in p.stdout
