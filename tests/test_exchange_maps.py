"""The x passes' exchange maps, chosen at compile time by a bank simulation
(xpass_warp.cuh), checked on the host: every map is a bijection into its
group's buffer and every stage boundary of every x plan is conflict-free."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "wavedm.jl_gb300", "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")


def test_exchange_maps_are_conflict_free_bijections(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "exchange_maps_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-I", CSRC, "-I", INCLUDE, os.path.join(HERE, "exchange_maps_check.cu"),
                    "-o", exe], check=True, capture_output=True, timeout=600)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    lines = r.stdout.strip().splitlines()
    assert r.returncode == 0, r.stdout
    assert lines[-1] == "ALL OK"
    assert len(lines) >= 20  # one line per stage boundary of the 12 plans
