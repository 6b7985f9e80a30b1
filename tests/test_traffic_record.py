"""The ncu traffic record that bench.py reports as roofline.traffic (CPU).

bench.py reads per-pass DRAM bytes from a committed capture and marks them
valid only while the kernel sources hash to the key stored with the capture.
The key ignores comments and blank space, so a comment edit keeps the record
and any code edit invalidates it.
"""
import json
import os
import shutil
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _copy_csrc(tmp_path):
    dst = tmp_path / "csrc"
    shutil.copytree(bench.CSRC, dst)
    return dst


def test_source_hash_ignores_comments_and_follows_code(tmp_path):
    csrc = _copy_csrc(tmp_path)
    h0 = bench.kernel_source_hash(str(csrc))
    f = csrc / "passes.cuh"
    text = f.read_text(encoding="utf-8")
    f.write_text("// a new line comment\n/* a block\n comment */\n\n" + text.replace("\n", "\n\n", 3),
                 encoding="utf-8")
    assert bench.kernel_source_hash(str(csrc)) == h0
    f.write_text(text + "\nnamespace wdm { constexpr int kUnused = 1; }\n", encoding="utf-8")
    assert bench.kernel_source_hash(str(csrc)) != h0


def test_host_pipeline_is_outside_the_key(tmp_path):
    """wdm_api.cu schedules the launches but holds no kernel: its edits keep the record."""
    csrc = _copy_csrc(tmp_path)
    h0 = bench.kernel_source_hash(str(csrc))
    api = csrc / "wdm_api.cu"
    api.write_text(api.read_text(encoding="utf-8") + "\nstatic int unused_host_value = 0;\n", encoding="utf-8")
    assert bench.kernel_source_hash(str(csrc)) == h0


def test_record_covers_every_pass_of_the_step():
    with open(bench.TRAFFIC_FILE) as fh:
        cap = json.load(fh)
    assert len(cap["kernel_source_hash"]) == 16
    assert "--clock-control none" in cap["command"]
    passes = cap["passes"]
    for name in ("kick_xfft_fwd/staged", "kick_final/staged", "psi_y_fwd/tma", "psi_z_drift/tma",
                 "psi_y_inv/tma", "psi_x_inv_rho/staged", "rho_y_fwd/tma", "rho_z_poisson/tma", "phi_y_inv/tma"):
        assert passes[name] > 0, name
    # no pass moves more DRAM bytes than its algorithmic bytes at 384^3
    # (16 B per cell of psi or of the half spectrum H, plus the rows the
    # x passes read or write besides)
    nc, nh = 384 ** 3, 193 * 384 * 384
    assert passes["psi_z_drift/tma"] <= 16 * nc
    assert passes["rho_z_poisson/tma"] <= 16 * nh
    assert passes["kick_xfft_fwd/staged"] <= 16 * nc + 8 * nh


def test_bench_marks_the_record_against_the_sources():
    sched = {k: {"impl": v} for k, v in (("x_kick", "staged"), ("psi_z", "tma"))}
    v, src = bench.ncu_traffic("psi_z_drift", 384, 3, sched)
    assert v > 0 and isinstance(src, dict)
    assert src["kernels_unchanged_since_capture"] == (
        json.load(open(bench.TRAFFIC_FILE))["kernel_source_hash"] == bench.kernel_source_hash())
    assert bench.ncu_traffic("psi_z_drift", 256, 3, sched)[0] is None
    assert bench.ncu_traffic("psi_y_fwd", 384, 3, sched)[0] is None  # its implementation not in sched
