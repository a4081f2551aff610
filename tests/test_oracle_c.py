"""The C oracle against the NumPy oracle, and against the reference's own C.

``oracle/fdtd_oracle.c`` (REAL=double, no FP contraction) must equal the
float64 NumPy restatement bit for bit; where the reference's C step functions
could be compiled here (``make -C oracle ref``), driving them directly must
give the same arrays too.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import ccore, fd1d, fd2d

DT = 0.01 / 6e8


def _fields(nx, ny, real=np.float64):
    return {k: np.zeros((nx, ny), dtype=real) for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy")}


@pytest.mark.parametrize("lossy,pml", [(True, True), (False, True), (False, False)])
def test_c_oracle_equals_numpy_2d(lossy, pml):
    nx, ny, ns, npml = 61, 47, 90, 7
    p = fd2d.pmlparam(nx, ny, npml, 0.333) if pml else None
    naz, nbz = fd2d.dielectric(nx, ny, npml, 10, DT, 30.0, 0.3) if lossy else (np.ones((nx, ny)), None)
    src = ("hard", nx // 2, ny // 2, ("gauss", 20, 6.0))
    st = fd2d.run(nx, ny, ns, pml=p, naz=naz, nbz=nbz, src=src, lossy=lossy, free_space_h=not pml)
    f = _fields(nx, ny)
    table = np.array([fd1d.gaussian(t, 20, 6.0) for t in range(1, ns + 1)])
    pd = None if p is None else {k: getattr(p, k) for k in ("fx1", "fx2", "fx3", "fy1", "fy2", "fy3",
                                                          "gx2", "gx3", "gy2", "gy3")}
    ccore.fd2d_steps(ccore.lib64(), np.float64, nx, ny, 0, ns, pd, naz, nbz if lossy else None,
                     (1, nx // 2, ny // 2), table, f if lossy else {k: v for k, v in f.items() if k != "iz"})
    keys = ["dz", "ez", "hx", "hy"] + (["iz"] if lossy else []) + (["ihx", "ihy"] if pml else [])
    for k in keys:
        np.testing.assert_array_equal(f[k], getattr(st, k), err_msg=k)


def test_c_oracle_equals_numpy_1d():
    nx, ns = 300, 500
    ca, cb = fd1d.dielectric_cacb(nx, DT, 4.0, 0.04)
    freq = np.array([1e8, 3e8, 7e8])
    st = fd1d.run(nx, ns, "cacb", ca=ca, cb=cb, src_kind="soft", src_k=5, wave=("gauss", 40, 12.0),
                  freq=freq, dt=DT, probes=(20, 250))
    lib = ccore.lib64()
    ex, hy, bc = np.zeros(nx), np.zeros(nx), np.zeros(4)
    table = np.array([fd1d.gaussian(t, 40, 12.0) for t in range(1, ns + 1)])
    dc = np.array([fd1d.dft_phase(t, freq, DT)[0] for t in range(1, ns + 1)])
    ds = np.array([fd1d.dft_phase(t, freq, DT)[1] for t in range(1, ns + 1)])
    pk = np.array([20, 250], dtype=np.int32)
    rp, ip = np.zeros((2, 3)), np.zeros((2, 3))
    p = lambda a: None if a is None else a.ctypes.data  # noqa: E731
    lib.oracle_fd1d_steps(nx, 1, 0, ns, p(ca), p(cb), None, None, None, None, 2, 5, p(table), 1, p(ex), p(hy),
                          None, None, None, p(bc), 3, p(dc), p(ds), 2, p(pk), p(rp), p(ip))
    np.testing.assert_array_equal(ex, st.ex)
    np.testing.assert_array_equal(hy, st.hy)
    np.testing.assert_array_equal(rp, st.r_pr)
    np.testing.assert_array_equal(ip, st.i_pr)


class _Pml(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("fx1", "fx2", "fx3", "fy1", "fy2", "fy3", "gx2", "gx3", "gy2", "gy3")]


class _Medium(C.Structure):
    _fields_ = [("naz", C.c_void_p), ("nbz", C.c_void_p)]


def test_reference_c_2d_equals_oracle():
    """fd2d/clang/fd2d_3_4.c's own dfield/efield/hfield (compiled from the
    reference sources into oracle/_ref) driven on a small grid."""
    ref = ccore.ref("fd2d_3_4")
    if ref is None:
        pytest.skip("reference C not compiled here (needs the reference checkout)")
    nx, ny, ns, npml = 40, 36, 70, 6
    p = fd2d.pmlparam(nx, ny, npml)
    naz, nbz = fd2d.dielectric(nx, ny, npml, 8, DT, 30.0, 0.3)
    st = fd2d.run(nx, ny, ns, pml=p, naz=naz, nbz=nbz, src=("hard", nx // 2, ny // 2, ("gauss", 20, 6.0)))
    f = _fields(nx, ny)
    vec = {k: np.ascontiguousarray(getattr(p, k)) for k in _Pml._fields_ and [n for n, _ in _Pml._fields_]}
    pml = _Pml(**{k: v.ctypes.data for k, v in vec.items()})
    naz_c, nbz_c = np.ascontiguousarray(naz), np.ascontiguousarray(nbz)
    md = _Medium(naz_c.ctypes.data, nbz_c.ctypes.data)
    ezi = np.zeros(ny)
    dp = C.c_void_p
    ref.dfield.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(_Pml), dp, dp, dp, dp]
    ref.efield.argtypes = [C.c_int, C.c_int, C.POINTER(_Medium), dp, dp, dp]
    ref.hfield.argtypes = [C.c_int, C.c_int, C.POINTER(_Pml), dp, dp, dp, dp, dp]
    for t in range(1, ns + 1):
        ref.dfield(t, nx, ny, C.byref(pml), ezi.ctypes.data, f["dz"].ctypes.data, f["hx"].ctypes.data,
                   f["hy"].ctypes.data)
        f["dz"][nx // 2, ny // 2] = fd1d.gaussian(t, 20, 6.0)
        ref.efield(nx, ny, C.byref(md), f["dz"].ctypes.data, f["iz"].ctypes.data, f["ez"].ctypes.data)
        ref.hfield(nx, ny, C.byref(pml), f["ez"].ctypes.data, f["ihx"].ctypes.data, f["ihy"].ctypes.data,
                   f["hx"].ctypes.data, f["hy"].ctypes.data)
    for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
        np.testing.assert_array_equal(f[k], getattr(st, k), err_msg=k)


def test_reference_c_1d_equals_oracle():
    """fd1d/clang/fd1d_1_3.c's exfield/hyfield (soft Gaussian at ex[1] computed by
    the C program itself) against the NumPy restatement of fd1d_1_3."""
    ref = ccore.ref("fd1d_1_3")
    if ref is None:
        pytest.skip("reference C not compiled here (needs the reference checkout)")
    kw = fd1d.program("fd1d_1_3")
    st = fd1d.run(**kw)
    nx = kw["nx"]
    cb = np.ascontiguousarray(kw["cb"])
    ex, hy, bc = np.zeros(nx), np.zeros(nx), np.zeros(4)
    dp = C.c_void_p
    ref.exfield.argtypes = [C.c_int, C.c_int, dp, dp, dp]
    ref.hyfield.argtypes = [C.c_int, dp, dp, dp]
    for t in range(1, kw["ns"] + 1):
        ref.exfield(t, nx, cb.ctypes.data, ex.ctypes.data, hy.ctypes.data)
        ref.hyfield(nx, ex.ctypes.data, hy.ctypes.data, bc.ctypes.data)
    # the C gaussian evaluates exp(-0.5*(t-t0)/s*(t-t0)/s): last-bit differences only
    np.testing.assert_allclose(ex, st.ex, rtol=0, atol=1e-13)
    np.testing.assert_allclose(hy, st.hy, rtol=0, atol=1e-13)
