"""The C-ABI library loads, exports every symbol include/fdtd.h declares, and
rejects bad arguments on the host before any launch (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

from tests.conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from simulation_gb300 import build
    build.build()
    from simulation_gb300 import _lib
    return _lib.lib()


def _declared():
    src = open(os.path.join(ROOT, "include", "fdtd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\**\s+\**((?:fdtd|fno)[a-z0-9_]*)\s*\(", src,
                                 flags=re.M)))


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/fdtd.h but not exported"
    from simulation_gb300 import _lib
    assert set(_lib.declared_symbols()) <= set(names) | {"fdtd_version"}


def test_status_strings(lib):
    assert lib.fdtd_version() >= 100
    assert lib.fdtd_status_string(0) == b"ok"
    assert lib.fdtd_status_to_error(1) == -6
    assert lib.fdtd_status_to_error(2) == -7
    assert lib.fdtd_status_to_error(0) == 0


def test_argument_checks_without_gpu(lib):
    """Every check runs on the host before any CUDA call, so bad arguments are
    reported even on a machine with no GPU."""
    from simulation_gb300 import _lib
    p = _lib.Params2D()
    s = _lib.State2D()
    assert lib.fdtd2d_step_n(None, None, 0, 1, 0, None, 0, None) == -1
    p.nx, p.ny = 2, 64
    assert lib.fdtd2d_step_n(C.byref(p), C.byref(s), 0, 1, 0, None, 0, None) == -2
    p.nx, p.ny = 64, 64
    assert lib.fdtd2d_step_n(C.byref(p), C.byref(s), 0, 1, 0, None, 0, None) == -1  # NULL fields
    fake = 0x10000  # never dereferenced: the calls below fail their checks first
    for k in ("dz", "ez", "hx", "hy"):
        setattr(s, k, fake)
    p.naz = fake
    p.pml.fx1 = fake  # 1 of 10 PML pointers
    assert lib.fdtd2d_step_n(C.byref(p), C.byref(s), 0, 1, 0, None, 0, None) == -1
    p.pml.fx1 = None
    p.src.kind, p.src.i, p.src.j = 1, 70, 3
    assert lib.fdtd2d_step_n(C.byref(p), C.byref(s), 0, 1, 0, None, 0, None) == -4
    p.src.i = 3
    p.src.table, p.src.table_len = fake, 5
    assert lib.fdtd2d_step_n(C.byref(p), C.byref(s), 0, 10, 0, None, 0, None) == -2  # table too short
    assert lib.fdtd2d_step_n(C.byref(p), C.byref(s), 0, 2, 9, None, 0, None) == -4  # steps per pass
    assert lib.fdtd2d_step_n(C.byref(p), C.byref(s), -1, 2, 0, None, 0, None) == -4
    q = _lib.Params1D()
    t = _lib.State1D()
    q.nx = 3
    assert lib.fdtd1d_step_n(C.byref(q), C.byref(t), 0, 1, None) == -2
    q.nx, q.form = 64, 7
    t.ex = t.hy = fake
    assert lib.fdtd1d_step_n(C.byref(q), C.byref(t), 0, 1, None) == -4
    q.form = 0
    assert lib.fdtd1d_step_n(C.byref(q), C.byref(t), 0, 1, None) == -1  # cb missing
    assert lib.fdtd2d_dielectric_cylinder(64, 64, 40, 10.0, 1e-11, 30.0, 0.3, fake, fake, None) == -2


def test_surrogate_and_gemm_argument_checks_without_gpu(lib):
    """The surrogate helpers and the tensor-core GEMM validate on the host too."""
    from simulation_gb300 import _lib
    fake = C.c_void_p(0x10000)
    d = C.c_double
    # propagation frame: NULL pointers, then bad sizes (nf > 64, n < 1, negative probes)
    assert lib.fno_propagation(4, 2048, None, 64, fake, d(8.0), d(0.05), d(1.0), 30, 10, fake, None) == -1
    assert lib.fno_propagation(4, 2048, fake, 65, fake, d(8.0), d(0.05), d(1.0), 30, 10, fake, None) == -2
    assert lib.fno_propagation(0, 2048, fake, 64, fake, d(8.0), d(0.05), d(1.0), 30, 10, fake, None) == -2
    assert lib.fno_propagation(4, 2048, fake, 64, fake, d(8.0), d(0.05), d(1.0), -1, 10, fake, None) == -2
    assert lib.fno_propagation(4, 2048, fake, 64, fake, d(0.0), d(0.05), d(1.0), 30, 10, fake, None) == -2
    assert lib.fno_cmul(4, 64, None, fake, 0, fake, None) == -1
    assert lib.fno_cmul(0, 64, fake, fake, 0, fake, None) == -2
    # lift: at most 8 input channels
    assert lib.fno_lift_fwd(16, 128, 9, fake, fake, fake, fake, None) == -2
    assert lib.fno_lift_bwd(16, 128, 0, fake, fake, fake, fake, None) == -2
    assert lib.fno_rel_mse(4, 128, C.c_float(0.0), fake, fake, fake, fake, None) == -2
    # GEMM descriptor: NULL, then a non-16-byte-aligned leading dimension
    assert lib.fdtd_gemm_bf16(None, None, None) == -1
    g = _lib.GemmDesc()
    g.M, g.N, g.K, g.batch = 128, 128, 64, 1
    g.A, g.B, g.C32 = 0x10000, 0x10000, 0x10000
    g.lda, g.ldb, g.ldc = 65, 64, 128  # 65 BF16 = 130 bytes per row
    assert lib.fdtd_gemm_bf16(C.byref(g), None, None) < 0


def test_workspace_size_host_arithmetic(lib):
    """fdtd2d_workspace_size is host arithmetic: the ping-pong field slots
    (256-byte rounded), plus 64 incident-line rows of ny floats and 64 (hxi,
    hxi) pairs with TF/SF on; 0 where the fused pass does not apply."""
    from simulation_gb300 import _lib
    lib.fdtd2d_workspace_size.restype = C.c_size_t
    p = _lib.Params2D()
    fake = 0x10000
    p.nx, p.ny = 100, 96
    slot = (100 * 96 * 4 + 255) // 256 * 256
    assert lib.fdtd2d_workspace_size(C.byref(p), 0) == 3 * slot  # lossless, no PML
    p.nbz = fake
    for k, _ in _lib.Pml2D._fields_:
        setattr(p.pml, k, fake)
    assert lib.fdtd2d_workspace_size(C.byref(p), 0) == 6 * slot  # lossy + PML
    p.nf = 3  # the DFT needs no tables of its own
    assert lib.fdtd2d_workspace_size(C.byref(p), 0) == 6 * slot
    p.tfsf_npml = 8
    line = (64 * 96 * 4 + 255) // 256 * 256 + 512
    assert lib.fdtd2d_workspace_size(C.byref(p), 0) == 6 * slot + line
    p.nf = 9  # beyond the fused pass's frequencies: three launches, no workspace
    assert lib.fdtd2d_workspace_size(C.byref(p), 0) == 0
    p.nf = 3
    p.ny = 98  # ny % 4 != 0
    assert lib.fdtd2d_workspace_size(C.byref(p), 0) == 0
    p.ny = 16388  # TF/SF line beyond the shared-memory limit
    assert lib.fdtd2d_workspace_size(C.byref(p), 0) == 0
    p.tfsf_npml = 0
    assert lib.fdtd2d_workspace_size(C.byref(p), 0) == 6 * ((100 * 16388 * 4 + 255) // 256 * 256)


def test_adjoint_and_noalloc_argument_checks_without_gpu(lib):
    """The one-call adjoint's workspace size is host arithmetic (checkpoint
    states, pass ping-pong, two record buffers, adjoint ping-pong), and it and
    the no-alloc step reject bad arguments before any CUDA call."""
    from simulation_gb300 import _lib
    fake = 0x10000  # never dereferenced
    p = _lib.Params2D()
    p.nx, p.ny = 64, 64
    p.naz = fake
    for k, _ in _lib.Pml2D._fields_:
        setattr(p.pml, k, fake)
    a = _lib.AdjointParams2D(100, 16, 40, 32, 2.0, _lib.Box2D(20, 20, 16, 16))
    slot = (64 * 64 * 4 + 255) // 256 * 256
    ncp = -(-100 // 16)
    size = lib.fdtd2d_tm_adjoint_workspace_size
    # lossless: 5 fields per state, 3 per record (dz, hx, hy)
    assert size(C.byref(p), C.byref(a)) == slot * ((ncp + 1) * 5 + 2 * 5 + 1 + 2 * 15 * 3 + 2 * 5 + 1)
    p.nbz = fake  # lossy: iz too
    assert size(C.byref(p), C.byref(a)) == slot * ((ncp + 1) * 6 + 2 * 6 + 1 + 2 * 15 * 4 + 2 * 6 + 1)
    bad = [("ny", 66), ("nsteps", 0), ("checkpoint", 0), ("probe_i", 64), ("tfsf_npml", 8), ("nf", 2)]
    for name, v in bad:
        obj = a if hasattr(a, name) else p
        old = getattr(obj, name)
        setattr(obj, name, v)
        assert size(C.byref(p), C.byref(a)) == 0, name
        setattr(obj, name, old)
    a.box = _lib.Box2D(60, 20, 16, 16)  # past the grid
    assert size(C.byref(p), C.byref(a)) == 0
    a.box = _lib.Box2D(20, 20, 16, 16)
    p.src.kind, p.src.i, p.src.j = 1, 30, 30  # a source needs its table, long enough
    assert size(C.byref(p), C.byref(a)) == 0
    p.src.table, p.src.table_len = fake, 99
    assert size(C.byref(p), C.byref(a)) == 0
    p.src.table_len = 100
    n = size(C.byref(p), C.byref(a))
    assert n > 0
    fwd, rev = lib.fdtd2d_tm_adjoint_forward, lib.fdtd2d_tm_adjoint_reverse
    assert fwd(C.byref(p), C.byref(a), None, None, fake, n, None) == -1  # no trace buffer
    assert fwd(C.byref(p), C.byref(a), fake, None, None, n, None) == -9  # no workspace
    assert fwd(C.byref(p), C.byref(a), fake, None, fake + 16, n, None) == -3  # workspace not 256-byte aligned
    assert fwd(C.byref(p), C.byref(a), fake, None, fake, n - 1, None) == -9  # workspace too small
    assert rev(C.byref(p), C.byref(a), None, None, fake, n, None) == -1  # no gradient buffer
    p.nbz = None
    assert rev(C.byref(p), C.byref(a), fake, fake, fake, n, None) == -4  # dJ/dnbz of a lossless box
    # no-alloc step: bad step counts and grids past its static array
    s = _lib.State2D()
    assert lib.fdtd2d_step_n_noalloc(C.byref(p), C.byref(s), 0, -1, 0, None) == -4
    assert lib.fdtd2d_step_n_noalloc(C.byref(p), C.byref(s), -1, 1, 0, None) == -4
    p.nx, p.ny = 1025, 1024
    assert lib.fdtd2d_step_n_noalloc(C.byref(p), C.byref(s), 0, 1, 0, None) == -2
