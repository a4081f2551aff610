"""Float64 NumPy restatement of the reference's 1D FDTD programs (oracle only).

The reference (dsarvan/simulation, ``fd1d/program``) writes each chapter-1/2
program as a stand-alone script.  This module restates their time loop as one
parametrised driver so the GPU path can be compared with any of them:

* ``form="cb"``    -- ``ex[1:nx] += cb*(hy[i-1]-hy[i])``        fd1d/program/fd1d_1_3.py:55
* ``form="cacb"``  -- ``ex = ca*ex + cb*(hy[i-1]-hy[i])``       fd1d/program/fd1d_1_5.py:65
* ``form="dform"`` -- ``dx += 0.5*curl; ex = nax*(dx-ix); ix += nbx*ex``
                                                              fd1d/program/fd1d_2_2.py:74-84
* ``form="debye"`` -- D-form plus the Debye ``sx`` recursion   fd1d/program/fd1d_2_3.py:82-86

Step order follows the reference exactly:

* chapter-1 forms (fd1d/program/fd1d_1_3.py:53-62): E update, source, ABC, H;
* chapter-2 forms (fd1d/program/fd1d_2_2.py:138-142): D update + source
  (``dxfield``), E from D (``exfield``), running DFT (``fourier``), then ABC
  and H (``hyfield``).
"""
from __future__ import annotations

import numpy as np
from numpy import pi, cos, sin

EPS0 = 8.854e-12  # vacuum permittivity (F/m), fd1d/program/fd1d_1_5.py:40


def gaussian(t: int, t0: float, spread: float) -> float:
    """fd1d/program/fd1d_1_1.py:27-28."""
    return float(np.exp(-0.5 * ((t - t0) / spread) ** 2))


def sinusoidal(t: int, ds: float, freq: float) -> float:
    """fd1d/program/fd1d_1_4.py:30-32 (dt = ds/6e8)."""
    dt = ds / 6e8
    return float(np.sin(2 * np.pi * freq * dt * t))


def source_value(t: int, wave: tuple) -> float:
    """``wave`` is ("gauss", t0, spread) or ("sin", ds, freq)."""
    if wave[0] == "gauss":
        return gaussian(t, wave[1], wave[2])
    if wave[0] == "sin":
        return sinusoidal(t, wave[1], wave[2])
    raise ValueError(f"unknown waveform {wave!r}")


def dielectric_cb(nx: int, epsr: float, start: int | None = None) -> np.ndarray:
    """fd1d/program/fd1d_1_3.py:31-34: cb = 0.5, and 0.5/epsr from ``start`` (nx//2)."""
    cb = 0.5 + np.zeros(nx, dtype=np.float64)
    cb[(nx // 2 if start is None else start):] = 0.5 / epsr
    return cb


def dielectric_cacb(nx: int, dt: float, epsr: float, sigma: float, start: int | None = None):
    """fd1d/program/fd1d_1_5.py:37-44."""
    ca = 1.0 + np.zeros(nx, dtype=np.float64)
    cb = 0.5 + np.zeros(nx, dtype=np.float64)
    epsf = dt * sigma / (2 * EPS0 * epsr)
    s = nx // 2 if start is None else start
    ca[s:] = (1 - epsf) / (1 + epsf)
    cb[s:] = 0.5 / (epsr * (1 + epsf))
    return ca, cb


def dielectric_dform(nx: int, dt: float, epsr: float, sigma: float, start: int | None = None):
    """fd1d/program/fd1d_2_2.py:95-103 -> (nax, nbx)."""
    nax = np.full(nx, 1.0, dtype=np.float64)
    nbx = np.full(nx, 0.0, dtype=np.float64)
    s = nx // 2 if start is None else start
    nax[s:] = 1 / (epsr + sigma * dt / EPS0)
    nbx[s:] = sigma * dt / EPS0
    return nax, nbx


def dielectric_debye(nx: int, dt: float, chi: float, tau: float, epsr: float, sigma: float,
                     start: int | None = None):
    """fd1d/program/fd1d_2_3.py:97-109 -> (nax, nbx, ncx, ndx)."""
    nax = np.full(nx, 1.0, dtype=np.float64)
    nbx = np.full(nx, 0.0, dtype=np.float64)
    ncx = np.full(nx, 0.0, dtype=np.float64)
    ndx = np.full(nx, 0.0, dtype=np.float64)
    s = nx // 2 if start is None else start
    nax[s:] = 1 / (epsr + sigma * dt / EPS0 + chi * dt / tau)
    nbx[s:] = sigma * dt / EPS0
    ncx[s:] = np.exp(-dt / tau)
    ndx[s:] = chi * dt / tau
    return nax, nbx, ncx, ndx


class State1D:
    """Field arrays of one 1D program (all float64, zero-initialised)."""

    def __init__(self, nx: int, nf: int = 0, probes: int = 0, full_dft: bool = False):
        self.ex = np.zeros(nx)
        self.hy = np.zeros(nx)
        self.dx = np.zeros(nx)
        self.ix = np.zeros(nx)
        self.sx = np.zeros(nx)
        self.bc = np.zeros(4)
        self.r_pt = np.zeros((nf, nx)) if full_dft else None
        self.i_pt = np.zeros((nf, nx)) if full_dft else None
        # probe DFT accumulators, [nprobe][nf]
        self.r_pr = np.zeros((probes, nf))
        self.i_pr = np.zeros((probes, nf))


def abc(ex: np.ndarray, bc: np.ndarray, nx: int) -> None:
    """Two-step-back absorbing boundary, fd1d/program/fd1d_1_2.py:47-48."""
    ex[0], bc[0], bc[1] = bc[0], bc[1], ex[1]
    ex[nx - 1], bc[3], bc[2] = bc[3], bc[2], ex[nx - 2]


def dft_phase(t: int, freq: np.ndarray, dt: float):
    """cos/sin factors of fd1d/program/fd1d_2_2.py:65-71 (argument 2*pi*f*dt*t)."""
    arg = 2 * pi * freq * dt * t
    return cos(arg), sin(arg)


def run(nx: int, ns: int, form: str = "cb", *, cb=None, ca=None, nax=None, nbx=None,
        ncx=None, ndx=None, src_kind: str = "soft", src_k: int = 1,
        wave: tuple = ("gauss", 40, 12.0), abc_on: bool = True,
        freq=None, dt: float = 0.01 / 6e8, probes=(), full_dft: bool = False,
        state: State1D | None = None, t_start: int = 1) -> State1D:
    """Run ``ns`` steps (t = t_start .. t_start+ns-1) of one 1D program.

    ``src_kind`` is "hard" (``ex[k] = v``, fd1d/program/fd1d_1_1.py:43) or
    "soft" (``ex[k] += v``, fd1d/program/fd1d_1_3.py:57); in the D forms the
    source goes into ``dx`` (fd1d/program/fd1d_2_2.py:78).  ``probes`` lists
    cells whose running DFT is accumulated (the reference's input probe is
    ``ex[10]``, fd1d/program/fd1d_2_2.py:67); ``full_dft`` also accumulates
    every cell (``r_pt/i_pt``, :70-71).
    """
    freq = np.zeros(0) if freq is None else np.asarray(freq, dtype=np.float64).reshape(-1)
    nf = freq.size
    st = state or State1D(nx, nf, len(probes), full_dft)
    ex, hy, dx, ix, sx, bc = st.ex, st.hy, st.dx, st.ix, st.sx, st.bc
    for t in range(t_start, t_start + ns):
        v = source_value(t, wave)
        if form in ("cb", "cacb"):
            if form == "cb":
                ex[1:nx] += cb[1:nx] * (hy[0:nx - 1] - hy[1:nx])
            else:
                ex[1:nx] = ca[1:nx] * ex[1:nx] + cb[1:nx] * (hy[0:nx - 1] - hy[1:nx])
            if src_kind == "hard":
                ex[src_k] = v
            elif src_kind == "soft":
                ex[src_k] += v
        elif form in ("dform", "debye"):
            dx[1:nx] += 0.5 * (hy[0:nx - 1] - hy[1:nx])
            if src_kind == "hard":
                dx[src_k] = v
            elif src_kind == "soft":
                dx[src_k] += v
            if form == "dform":
                ex[1:nx] = nax[1:nx] * (dx[1:nx] - ix[1:nx])
                ix[1:nx] += nbx[1:nx] * ex[1:nx]
            else:
                ex[1:nx] = nax[1:nx] * (dx[1:nx] - ix[1:nx] - ncx[1:nx] * sx[1:nx])
                ix[1:nx] += nbx[1:nx] * ex[1:nx]
                sx[1:nx] = ncx[1:nx] * sx[1:nx] + ndx[1:nx] * ex[1:nx]
        else:
            raise ValueError(form)
        if nf:
            # running DFT after the E stage and before the ABC, as
            # fd1d/program/fd1d_2_2.py:138-142 orders fourier() and hyfield()
            c, s = dft_phase(t, freq, dt)
            for p, k in enumerate(probes):
                st.r_pr[p] += c * ex[k]
                st.i_pr[p] -= s * ex[k]
            if full_dft:
                st.r_pt += c[:, None] * ex[None, :]
                st.i_pt -= s[:, None] * ex[None, :]
        if abc_on:
            abc(ex, bc, nx)
        hy[0:nx - 1] += 0.5 * (ex[0:nx - 1] - ex[1:nx])
    return st


def amplitude_phase(r_pt, i_pt, r_in, i_in):
    """fd1d/program/fd1d_2_2.py:145-146."""
    amplt = 1 / np.hypot(r_in, i_in) * np.hypot(r_pt, i_pt)
    phase = np.arctan2(i_pt, r_pt) - np.arctan2(i_in, r_in)
    return amplt, phase


# ---------------------------------------------------------------- programs
# Parameters of each reference program's main(), so tests can replay them.

def program(name: str) -> dict:
    """Keyword arguments of ``run`` that replay a reference program's main()."""
    ds = 0.01
    dt = ds / 6e8
    if name == "fd1d_1_1":   # fd1d/program/fd1d_1_1.py:33-45
        return dict(nx=512, ns=300, form="cb", cb=np.full(512, 0.5), src_kind="hard",
                    src_k=256, wave=("gauss", 40, 12.0), abc_on=False)
    if name == "fd1d_1_2":   # fd1d/program/fd1d_1_2.py
        return dict(nx=512, ns=570, form="cb", cb=np.full(512, 0.5), src_kind="hard",
                    src_k=256, wave=("gauss", 40, 12.0), abc_on=True)
    if name == "fd1d_1_3":   # fd1d/program/fd1d_1_3.py:40-62
        return dict(nx=512, ns=740, form="cb", cb=dielectric_cb(512, 4.0), src_kind="soft",
                    src_k=1, wave=("gauss", 40, 12.0), abc_on=True)
    if name == "fd1d_1_4":   # fd1d/program/fd1d_1_4.py:41-65
        return dict(nx=512, ns=740, form="cb", cb=dielectric_cb(512, 4.0), src_kind="soft",
                    src_k=1, wave=("sin", 0.01, 700e6), abc_on=True)
    if name == "fd1d_1_5":   # fd1d/program/fd1d_1_5.py:47-72
        ca, cb = dielectric_cacb(512, dt, 4.0, 0.04)
        return dict(nx=512, ns=740, form="cacb", ca=ca, cb=cb, src_kind="soft", src_k=1,
                    wave=("sin", 0.01, 700e6), abc_on=True)
    if name == "fd1d_2_1":   # fd1d/program/fd1d_2_1.py
        nax, nbx = dielectric_dform(512, dt, 4.0, 0.04)
        return dict(nx=512, ns=740, form="dform", nax=nax, nbx=nbx, src_kind="soft",
                    src_k=1, wave=("sin", 0.01, 700e6), abc_on=True)
    if name == "fd1d_2_2":   # fd1d/program/fd1d_2_2.py:106-142
        nax, nbx = dielectric_dform(512, dt, 4.0, 0.0)
        return dict(nx=512, ns=740, form="dform", nax=nax, nbx=nbx, src_kind="soft",
                    src_k=1, wave=("gauss", 50, 10.0), abc_on=True,
                    freq=np.array([100e6, 200e6, 500e6]), dt=dt, probes=(10,), full_dft=True)
    if name == "fd1d_2_3":   # fd1d/program/fd1d_2_3.py
        nax, nbx, ncx, ndx = dielectric_debye(512, dt, 2.0, 0.001e-6, 2.0, 0.01)
        return dict(nx=512, ns=740, form="debye", nax=nax, nbx=nbx, ncx=ncx, ndx=ndx,
                    src_kind="soft", src_k=1, wave=("gauss", 50, 10.0), abc_on=True,
                    freq=np.array([50e6, 200e6, 500e6]), dt=dt, probes=(10,), full_dft=True)
    if name == "problem_1_4":  # fd1d/problem/problem_1_4/fd1d_1_1.py:24-70 (soft source at k=5)
        cb = np.full(201, 0.5)
        cb[100:] = 0.5 / 4
        return dict(nx=201, ns=440, form="cb", cb=cb, src_kind="soft", src_k=5,
                    wave=("gauss", 40, 12), abc_on=True)
    if name == "config1":    # plain 1D dielectric case: ke=200, hard source at k=5, 1000 steps
        cb = np.full(200, 0.5)
        cb[100:] = 0.5 / 4
        return dict(nx=200, ns=1000, form="cb", cb=cb, src_kind="hard", src_k=5,
                    wave=("gauss", 40, 12.0), abc_on=True)
    raise KeyError(name)
