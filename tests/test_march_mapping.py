"""Warp -> work mapping of the fused pass with TF/SF, checked on the CPU.

The fused pass compiles the TF/SF edge logic only into the body that edge
warps run and halves their segments across extra warps.  The check program
(tests/march_mapping_check.cu) includes the kernel header, uses its own
tf_stripe / tf_segment predicates, and verifies over many grid shapes, PML
widths, segment lengths and steps per pass that every (stripe, row) is owned
exactly once and that no warp classified as plain reaches an edge cell.  It
is host code only: built with nvcc, run here, no GPU needed.
"""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT


def test_tfsf_edge_classification_and_coverage(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "march_mapping_check")
    cmd = [nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "simulation_gb300", "csrc"),
           os.path.join(ROOT, "tests", "march_mapping_check.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-2000:]
