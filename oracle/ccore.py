"""ctypes access to the C oracle (test infrastructure only).

``lib64()`` is the float64 restatement (bit-identical to the NumPy oracle),
``lib32()`` the float32 OpenMP build and ``lib32_native()`` the same built for
the host's CPU: the timed CPU baseline.
``ref(name)`` loads a reference C program compiled from its own sources
(``make -C oracle ref``), when that was possible.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_L = {}


def build(ref: bool = False) -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _load(name: str):
    if name not in _L:
        path = os.path.join(HERE, "_build", name)
        if not os.path.exists(path):
            build()
        h = C.CDLL(path)
        dp = C.c_void_p
        h.oracle_fd2d_steps.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, dp, dp, dp, C.c_int, C.c_int, C.c_int,
                                        dp, dp, dp, dp, dp, dp, dp, dp]
        h.oracle_fd2d_steps.restype = None
        h.oracle_fd1d_steps.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int] + [dp] * 6 + [C.c_int, C.c_int, dp,
                                        C.c_int] + [dp] * 6 + [C.c_int, dp, dp, C.c_int, dp, dp, dp]
        h.oracle_fd1d_steps.restype = None
        h.oracle_fd1d_batch.argtypes = [C.c_int] + [dp] * 6 + [C.c_int, dp, C.c_int, C.c_int, dp, dp, dp, dp, dp]
        h.oracle_fd1d_batch.restype = None
        h.oracle_set_threads.argtypes = [C.c_int]
        h.oracle_threads.restype = C.c_int
        _L[name] = h
    return _L[name]


def lib64():
    return _load("liboracle64.so")


def lib32():
    return _load("liboracle32.so")


def lib32_native():
    """The float32 port built for this host's CPU (-march/-mcpu=native), or
    None where the compiler could not build it.  Timing only."""
    if not os.path.exists(os.path.join(HERE, "_build", "liboracle32n.so")):
        build()
    if not os.path.exists(os.path.join(HERE, "_build", "liboracle32n.so")):
        return None
    return _load("liboracle32n.so")


def _p(a):
    return None if a is None else a.ctypes.data


def fd2d_steps(lib, real, nx, ny, t0, ns, pml, naz, nbz, src, src_table, f) -> None:
    """Advance fields ``f`` (dict of C-contiguous arrays of dtype ``real``) in place.

    ``pml``: dict of the ten vectors or None; ``src``: (kind 0/1/2, i, j);
    ``src_table``: float64 array, row t-1 for step t.
    """
    keep = []
    pml_arr = None
    if pml is not None:
        vecs = [np.ascontiguousarray(pml[k], dtype=real) for k in
                ("fx1", "fx2", "fx3", "fy1", "fy2", "fy3", "gx2", "gx3", "gy2", "gy3")]
        keep += vecs
        pml_arr = (C.c_void_p * 10)(*[v.ctypes.data for v in vecs])
    st = np.ascontiguousarray(src_table, dtype=np.float64) if src_table is not None else np.zeros(1)
    lib.oracle_fd2d_steps(nx, ny, t0, ns, C.cast(pml_arr, C.c_void_p) if pml_arr is not None else None,
                          _p(naz), _p(nbz), src[0], src[1], src[2], _p(st), _p(f["dz"]), _p(f["ez"]),
                          _p(f.get("iz")), _p(f["hx"]), _p(f["hy"]), _p(f.get("ihx")), _p(f.get("ihy")))


def fd1d_steps(lib, real, nx, form, t0, ns, co, src_kind, src_k, src_table, abc, f) -> None:
    """Advance one 1D line in place: ``co`` maps ca/cb/nax/nbx/ncx/ndx to arrays
    of dtype ``real`` (absent ones None), ``f`` maps ex/hy/dx/ix/sx/bc likewise;
    ``src_table`` is float64, row t-1 for step t.  No DFT probes."""
    st = np.ascontiguousarray(src_table, dtype=np.float64) if src_table is not None else np.zeros(1)
    g = lambda k: _p(co.get(k))  # noqa: E731
    h = lambda k: _p(f.get(k))  # noqa: E731
    lib.oracle_fd1d_steps(nx, form, t0, ns, g("ca"), g("cb"), g("nax"), g("nbx"), g("ncx"), g("ndx"), src_kind,
                          src_k, _p(st), int(abc), h("ex"), h("hy"), h("dx"), h("ix"), h("sx"), h("bc"), 0, None,
                          None, 0, None, None, None)


def fd1d_batch(lib, real, ke, layer_off, layer_start, layer_end, layer_ca, layer_cb, src_k, src_table, ns,
               dcos, dsin, probe_in, probe_out):
    """Spectra accumulators [nruns][4][nf] (re_in, im_in, re_out, im_out)."""
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    ke, lo, ls, le, pi, po = i32(ke), i32(layer_off), i32(layer_start), i32(layer_end), i32(probe_in), i32(probe_out)
    lca, lcb, stb, dc, ds = f64(layer_ca), f64(layer_cb), f64(src_table), f64(dcos), f64(dsin)
    nf = dc.shape[1]
    spec = np.zeros((ke.size, 4, nf), dtype=real)
    lib.oracle_fd1d_batch(ke.size, _p(ke), _p(lo), _p(ls), _p(le), _p(lca), _p(lcb), src_k, _p(stb), ns, nf,
                          _p(dc), _p(ds), _p(pi), _p(po), _p(spec))
    return spec


def ref(name: str):
    """The reference's own compiled C program ``name`` (e.g. 'fd2d_3_4'), or None."""
    path = os.path.join(HERE, "_ref", f"libref_{name}.so")
    if not os.path.exists(path):
        return None
    return C.CDLL(path)
