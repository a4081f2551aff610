"""Warp -> work layout of the fused passes, checked on the CPU.

One launch is a single wave of warps; the stripes and segments that hold
the absorbing layer, the grid's edges or the TF/SF box's edge columns get
shorter work.  The check program (tests/march_mapping_check.cu) includes the
kernel header and calls its own plain_layout / plain_work over many grid
shapes, layer widths, TF/SF boxes, wave sizes, cost factors and steps per
pass: every (stripe, row) is owned by exactly one warp, every warp's work is
inside the grid, and every instantiation's shared memory fits a block.  It
is host code only: built with nvcc, run here, no GPU needed.
"""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT


def test_work_layout_coverage_and_shared_memory(tmp_path):
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
