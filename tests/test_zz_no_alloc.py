"""The allocation-free 2D entry point, fdtd2d_step_n_noalloc.

It serves callers that cannot allocate device memory: its workspace is a
static device array inside the library instead of a buffer the caller
passes.  Through the C-ABI, its results must equal the regular
fdtd2d_step_n's, on two calls in a row (the second on another grid, so the
array holds the first call's leftovers).  This file is collected last on
purpose, and passes alone in a fresh process as well as after the others.
"""
import ctypes as C

import pytest
import torch

FIELDS = ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy")


def _sim(nx, ny):
    from simulation_gb300 import fd2d as G
    dt = 0.01 / 6e8
    naz, nbz = G.dielectric(nx, ny, 8, min(nx, ny) // 4, dt, 30.0, 0.3)
    return G.SimTM2D(nx, ny, pml=G.pmlparam(nx, ny, 8, 0.333), naz=naz, nbz=nbz,
                     source=G.PointSource(nx // 2, ny // 2, ("gauss", 20, 6.0)), ns=256)


@pytest.mark.gpu
def test_noalloc_matches_step_n_twice(cuda_lib):
    lib = cuda_lib
    st = torch.cuda.current_stream().cuda_stream
    for call, (nx, ny, t0, n) in enumerate(((256, 256, 0, 37), (300, 264, 0, 23))):
        a = _sim(nx, ny)  # through fdtd2d_step_n_noalloc
        b = _sim(nx, ny)  # through fdtd2d_step_n with its own workspace
        ws = b.workspace()
        assert ws is not None
        rc = lib.fdtd2d_step_n_noalloc(C.byref(a._p), C.byref(a._s), t0, n, 0, st)
        assert rc == 0, f"call {call}: noalloc rc={rc}"
        rc = lib.fdtd2d_step_n(C.byref(b._p), C.byref(b._s), t0, n, 0, ws.data_ptr(), ws.numel(), st)
        assert rc == 0
        torch.cuda.synchronize()
        for k in FIELDS:
            assert torch.equal(getattr(a, k), getattr(b, k)), f"call {call}: {k} differs"
        assert float(a.ez.abs().max()) > 0.0


@pytest.mark.gpu
def test_noalloc_rejects_oversized_grid(cuda_lib):
    from simulation_gb300 import _lib
    p = _lib.Params2D()
    s = _lib.State2D()
    p.nx, p.ny = 2048, 1024  # 2^21 cells > FDTD2D_NOALLOC_MAX_CELLS
    assert cuda_lib.fdtd2d_step_n_noalloc(C.byref(p), C.byref(s), 0, 4, 0, None) == -2


@pytest.mark.gpu
@pytest.mark.parametrize("n", [256, 1024])
def test_noalloc_with_tfsf_and_dft(cuda_lib, n):
    """TF/SF and a 3-frequency DFT through the allocation-free entry: at 256^2
    the fused passes (the incident-line tables fit the static array beside the
    fields), at 1024^2 (the fields alone fill it) one three-launch step per
    call.  Both equal the per-function launches bit for bit."""
    from simulation_gb300 import fd2d as G
    dt = 0.01 / 6e8

    def make():
        naz, nbz = G.dielectric(n, n, 8, n // 8, dt, 30.0, 0.3)
        return G.SimTM2D(n, n, pml=G.pmlparam(n, n, 8), naz=naz, nbz=nbz, lossy=True, tfsf_npml=8,
                         freq=[50e6, 300e6, 700e6], dt=dt, ns=64)
    a, b = make(), make()
    st = torch.cuda.current_stream().cuda_stream
    rc = cuda_lib.fdtd2d_step_n_noalloc(C.byref(a._p), C.byref(a._s), 0, 21, 0, st)
    assert rc == 0, f"noalloc rc={rc}"
    b.step_per_function(21)
    torch.cuda.synchronize()
    for k in a.FIELDS:
        if getattr(a, k) is None:
            continue
        assert torch.equal(getattr(a, k), getattr(b, k)), f"{n}^2: {k} differs"
