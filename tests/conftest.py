"""Test configuration: the ``gpu`` marker and shared helpers.

``-m "not gpu"`` runs on any CPU machine (oracle vs golden fixtures, host
logic, C-ABI loading and argument checks, multi-process gloo tests);
``-m gpu`` runs the parity tests proper on a CUDA device through the C-ABI.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests through the C-ABI)")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        with np.load(os.path.join(GOLDEN, name)) as z:
            return {k: z[k] for k in z.files}
    return load


@pytest.fixture(scope="session")
def cuda_lib():
    """Build (if needed) and load the CUDA library; GPU tests only."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    from simulation_gb300 import build
    build.build()
    from simulation_gb300 import _lib
    return _lib.lib()


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def assert_parity(gpu, ref, tol=1e-5, what=""):
    """max|gpu-ref| <= tol*peak|ref| and relative L2 <= tol (spec tolerance)."""
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    peak = np.abs(ref).max()
    maxabs = np.abs(gpu - ref).max()
    rl2 = rel_l2(gpu, ref)
    assert maxabs <= tol * max(peak, 1e-30), f"{what}: max-abs {maxabs:.3e} > {tol}*peak {peak:.3e} (relL2 {rl2:.3e})"
    assert rl2 <= tol, f"{what}: rel-L2 {rl2:.3e} > {tol} (max-abs {maxabs:.3e}, peak {peak:.3e})"
    return maxabs / max(peak, 1e-30), rl2
