"""1D Ex/Hy FDTD on the GPU: host mirror of the reference's fd1d programs.

Forms, sources and boundary follow dsarvan/simulation ``fd1d/program``:

* ``"cb"``    ex += cb*(hy[i-1]-hy[i])                (fd1d_1_3.py:55)
* ``"cacb"``  ex = ca*ex + cb*(hy[i-1]-hy[i])         (fd1d_1_5.py:65)
* ``"dform"`` dx/ix with nax/nbx                       (fd1d_2_2.py:74-84)
* ``"debye"`` D-form plus Debye sx with ncx/ndx        (fd1d_2_3.py:82-86)

with hard/soft Gaussian or sinusoidal sources, the two-step-back ABC
(fd1d_1_2.py:47-48) and running-DFT probes (fd1d_2_2.py:65-71).  The
coefficient helpers (``dielectric_*``) reproduce the reference's float64
formulas on the host; fields and coefficients live in float32 CUDA tensors and
every update runs in ``libfdtd_gb300.so``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr
from .sources import dft_tables, to_device, wave_values

EPS0 = 8.854e-12  # fd1d/program/fd1d_1_5.py:40
FORMS = {"cb": _lib.FORM_CB, "cacb": _lib.FORM_CACB, "dform": _lib.FORM_DFORM, "debye": _lib.FORM_DEBYE}


def dielectric_cb(nx: int, epsr: float, start: int | None = None) -> np.ndarray:
    """fd1d/program/fd1d_1_3.py:31-34 (float64)."""
    cb = 0.5 + np.zeros(nx)
    cb[(nx // 2 if start is None else start):] = 0.5 / epsr
    return cb


def dielectric_cacb(nx: int, dt: float, epsr: float, sigma: float, start: int | None = None):
    """fd1d/program/fd1d_1_5.py:37-44 (float64)."""
    ca = 1.0 + np.zeros(nx)
    cb = 0.5 + np.zeros(nx)
    epsf = dt * sigma / (2 * EPS0 * epsr)
    s = nx // 2 if start is None else start
    ca[s:] = (1 - epsf) / (1 + epsf)
    cb[s:] = 0.5 / (epsr * (1 + epsf))
    return ca, cb


def dielectric_dform(nx: int, dt: float, epsr: float, sigma: float, start: int | None = None):
    """fd1d/program/fd1d_2_2.py:95-103 (float64)."""
    nax = np.full(nx, 1.0)
    nbx = np.full(nx, 0.0)
    s = nx // 2 if start is None else start
    nax[s:] = 1 / (epsr + sigma * dt / EPS0)
    nbx[s:] = sigma * dt / EPS0
    return nax, nbx


def dielectric_debye(nx: int, dt: float, chi: float, tau: float, epsr: float, sigma: float,
                     start: int | None = None):
    """fd1d/program/fd1d_2_3.py:97-109 (float64)."""
    nax = np.full(nx, 1.0)
    nbx = np.full(nx, 0.0)
    ncx = np.full(nx, 0.0)
    ndx = np.full(nx, 0.0)
    s = nx // 2 if start is None else start
    nax[s:] = 1 / (epsr + sigma * dt / EPS0 + chi * dt / tau)
    nbx[s:] = sigma * dt / EPS0
    ncx[s:] = np.exp(-dt / tau)
    ndx[s:] = chi * dt / tau
    return nax, nbx, ncx, ndx


class Sim1D:
    """One 1D program: coefficients, fields, source, ABC and DFT probes on the GPU."""

    def __init__(self, nx: int, form: str = "cb", *, cb=None, ca=None, nax=None, nbx=None, ncx=None, ndx=None,
                 src_kind: str = "soft", src_k: int = 1, wave: tuple = ("gauss", 40, 12.0), abc: bool = True,
                 freq=None, dt: float = 0.01 / 6e8, probes=(), full_dft: bool = False, ns: int = 1024,
                 device="cuda", check_finite: bool = True):
        if nx < 4:
            raise ValueError("nx must be >= 4")
        if len(probes) > _lib.MAX_PROBES:
            raise ValueError(f"at most {_lib.MAX_PROBES} probes")
        self.nx, self.form, self.device = nx, form, torch.device(device)
        self.src_kind = {"hard": _lib.SRC_HARD, "soft": _lib.SRC_SOFT, "none": _lib.SRC_NONE}[src_kind]
        self.src_k, self.wave, self.abc, self.dt = src_k, wave, abc, dt
        self.freq = None if freq is None else np.asarray(freq, dtype=np.float64).reshape(-1)
        self.probes = tuple(int(k) for k in probes)
        self.full_dft = full_dft
        dev = self.device
        co = lambda a: None if a is None else to_device(np.asarray(a, dtype=np.float64), dev)  # noqa: E731
        self.cb, self.ca, self.nax, self.nbx, self.ncx, self.ndx = co(cb), co(ca), co(nax), co(nbx), co(ncx), co(ndx)
        z = lambda *shape: torch.zeros(shape, dtype=torch.float32, device=dev)  # noqa: E731
        self.ex, self.hy = z(nx), z(nx)
        df = form in ("dform", "debye")
        self.dx = z(nx) if df else None
        self.ix = z(nx) if df else None
        self.sx = z(nx) if form == "debye" else None
        self.bc = z(4)
        nf = 0 if self.freq is None else self.freq.size
        self.r_pt = z(nf, nx) if (nf and full_dft) else None
        self.i_pt = z(nf, nx) if (nf and full_dft) else None
        self.r_pr = z(max(len(self.probes), 1), max(nf, 1)) if nf else None
        self.i_pr = z(max(len(self.probes), 1), max(nf, 1)) if nf else None
        self.status = torch.zeros(1, dtype=torch.int32, device=dev) if check_finite else None
        self.t = 0
        self._tables(ns)

    def _tables(self, ns: int) -> None:
        self._ns = ns
        self.src_table = to_device(wave_values(self.wave, 1, ns), self.device) if self.src_kind else None
        self.dft_cos = self.dft_sin = None
        if self.freq is not None:
            cs, sn = dft_tables(self.freq, self.dt, 1, ns)
            self.dft_cos, self.dft_sin = to_device(cs, self.device), to_device(sn, self.device)
        p = _lib.Params1D()
        p.nx, p.form = self.nx, FORMS[self.form]
        for k in ("ca", "cb", "nax", "nbx", "ncx", "ndx"):
            setattr(p, k, ptr(getattr(self, k)))
        p.src_kind, p.src_k = self.src_kind, self.src_k
        p.src_table, p.src_table_len = ptr(self.src_table), ns
        p.abc = int(self.abc)
        if self.freq is not None:
            p.nf = self.freq.size
            p.dft_cos, p.dft_sin, p.dft_table_len = ptr(self.dft_cos), ptr(self.dft_sin), ns
            p.nprobe = len(self.probes)
            for q, k in enumerate(self.probes):
                p.probe_k[q] = k
            p.full_dft = int(self.full_dft)
        s = _lib.State1D()
        for k in ("ex", "hy", "dx", "ix", "sx", "bc", "r_pt", "i_pt", "r_pr", "i_pr"):
            setattr(s, k, ptr(getattr(self, k)))
        s.status = ptr(self.status)
        self._p, self._s = p, s

    def _ensure(self, t_last: int) -> None:
        if t_last > self._ns:
            self._tables(max(t_last, 2 * self._ns))

    MAX_FUSED_NX = 65536  # FDTD1D_MAX_FUSED_NX

    def step(self, n: int = 1) -> None:
        """Advance n steps: one fused launch (one thread-block cluster) when the
        line fits on-chip, else one launch per reference function per step."""
        if n <= 0:
            return
        if self.nx > self.MAX_FUSED_NX:
            self.step_per_function(n)
            return
        self._ensure(self.t + n)
        call("fdtd1d_step_n", self._p, self._s, self.t, n, _lib.stream_ptr())
        self.t += n

    def step_per_function(self, n: int = 1) -> None:
        """The reference loop body with one launch per reference function."""
        self._ensure(self.t + n)
        st = _lib.stream_ptr()
        for t in range(self.t + 1, self.t + n + 1):
            call("fdtd1d_efield", t, self._p, self._s, st)
            if self.freq is not None:
                call("fdtd1d_fourier", t, self._p, self._s, st)
            call("fdtd1d_hfield", self._p, self._s, st)
        self.t += n

    def check(self) -> None:
        if self.status is None:
            return
        v = int(self.status.item())
        if v:
            raise _lib.FdtdError(_lib.lib().fdtd_status_to_error(v), f"Sim1D status word {v:#x}")

    def amplitude_phase(self, probe: int = 0):
        """(amp, phase) float64 [nf][nx] of the full-field DFT against probe
        ``probe`` as input (fd1d/program/fd1d_2_2.py:145-146, on the device)."""
        if self.r_pt is None:
            raise ValueError("amplitude_phase needs freq=... and full_dft=True")
        if not 0 <= probe < len(self.probes):
            raise ValueError("no such probe")
        from .output import amplitude_phase
        return amplitude_phase(self.r_pt, self.i_pt, self.r_pr[probe], self.i_pr[probe])

    def head(self, name: str = "ex", n: int = 50) -> str:
        """``print(ex[0:50])`` of the reference's benchmark twins (fd1d/program/test_1_3.py:70)."""
        from .output import head
        return head(getattr(self, name), n)

    def save(self, path: str, names=None) -> str:
        """Write the fields to an .npz archive (or .npy files in a directory)."""
        from .output import save
        return save(self, path, names)

    FIELDS = ("ex", "hy", "dx", "ix", "sx", "bc", "r_pt", "i_pt", "r_pr", "i_pr")

    def state_dict(self) -> dict:
        d = {k: getattr(self, k).clone() for k in self.FIELDS if getattr(self, k) is not None}
        d["t"] = self.t
        return d

    def load_state_dict(self, d: dict) -> None:
        for k in self.FIELDS:
            if getattr(self, k) is not None:
                getattr(self, k).copy_(d[k])
        self.t = int(d["t"])


def program(name: str, **kw) -> Sim1D:
    """A ``Sim1D`` set up like one of the reference's fd1d programs' main()."""
    ds = 0.01
    dt = ds / 6e8
    if name == "fd1d_1_1":
        return Sim1D(512, "cb", cb=np.full(512, 0.5), src_kind="hard", src_k=256, wave=("gauss", 40, 12.0),
                     abc=False, **kw)
    if name == "fd1d_1_2":
        return Sim1D(512, "cb", cb=np.full(512, 0.5), src_kind="hard", src_k=256, wave=("gauss", 40, 12.0), **kw)
    if name == "fd1d_1_3":
        return Sim1D(512, "cb", cb=dielectric_cb(512, 4.0), src_kind="soft", src_k=1, wave=("gauss", 40, 12.0),
                     **kw)
    if name == "fd1d_1_4":
        return Sim1D(512, "cb", cb=dielectric_cb(512, 4.0), src_kind="soft", src_k=1, wave=("sin", 0.01, 700e6),
                     **kw)
    if name == "fd1d_1_5":
        ca, cb = dielectric_cacb(512, dt, 4.0, 0.04)
        return Sim1D(512, "cacb", ca=ca, cb=cb, src_kind="soft", src_k=1, wave=("sin", 0.01, 700e6), **kw)
    if name == "fd1d_2_1":
        nax, nbx = dielectric_dform(512, dt, 4.0, 0.04)
        return Sim1D(512, "dform", nax=nax, nbx=nbx, src_kind="soft", src_k=1, wave=("sin", 0.01, 700e6), **kw)
    if name == "fd1d_2_2":
        nax, nbx = dielectric_dform(512, dt, 4.0, 0.0)
        return Sim1D(512, "dform", nax=nax, nbx=nbx, src_kind="soft", src_k=1, wave=("gauss", 50, 10.0),
                     freq=[100e6, 200e6, 500e6], dt=dt, probes=(10,), full_dft=True, **kw)
    if name == "fd1d_2_3":
        nax, nbx, ncx, ndx = dielectric_debye(512, dt, 2.0, 0.001e-6, 2.0, 0.01)
        return Sim1D(512, "debye", nax=nax, nbx=nbx, ncx=ncx, ndx=ndx, src_kind="soft", src_k=1,
                     wave=("gauss", 50, 10.0), freq=[50e6, 200e6, 500e6], dt=dt, probes=(10,), full_dft=True, **kw)
    if name == "config1":
        cb = np.full(200, 0.5)
        cb[100:] = 0.5 / 4
        return Sim1D(200, "cb", cb=cb, src_kind="hard", src_k=5, wave=("gauss", 40, 12.0), **kw)
    raise KeyError(name)


PROGRAM_STEPS = {"fd1d_1_1": 300, "fd1d_1_2": 570, "fd1d_1_3": 740, "fd1d_1_4": 740, "fd1d_1_5": 740,
                 "fd1d_2_1": 740, "fd1d_2_2": 740, "fd1d_2_3": 740, "config1": 1000}
