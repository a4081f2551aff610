"""Per-step source and DFT tables, computed on the host in float64.

The reference evaluates its sources once per step in float64
(``gaussian``: fd1d/program/fd1d_1_1.py:27-28, fd2d/python/fd2d_3_4.py:84-86;
``sinusoidal``: fd1d/program/fd1d_1_4.py:30-32, fd2d/python/fd2d_3_2.py:55-58)
and its running DFT factors as ``cos/sin(2*pi*freq*dt*t)``
(fd1d/program/fd1d_2_2.py:65-71).  The GPU library reads these values from a
device table (row t-1 for step t), so a whole time loop can be enqueued or
graph-captured without per-step host work.  Values are computed with the same
NumPy expressions as the reference and rounded once to float32.
"""
from __future__ import annotations

import numpy as np


def wave_values(wave: tuple, t_start: int, n: int) -> np.ndarray:
    """float64 values of ``wave`` for t = t_start .. t_start+n-1.

    ``wave`` = ("gauss", t0, spread) | ("dgauss", t0, spread) | ("sin", ds, freq)
    | ("zero",).  "dgauss" is the derivative-of-Gaussian pulse -u exp(-u^2/2),
    u = (t - t0)/spread (not a reference waveform): it carries no DC content,
    so a soft source leaves no static charge whose slow decay in lossy layers
    would outlast a finite run and bias its spectra.
    """
    out = np.zeros(n, dtype=np.float64)
    kind = wave[0]
    for k in range(n):
        t = t_start + k
        if kind == "gauss":
            out[k] = np.exp(-0.5 * ((t - wave[1]) / wave[2]) ** 2)
        elif kind == "dgauss":
            u = (t - wave[1]) / wave[2]
            out[k] = -u * np.exp(-0.5 * u * u)
        elif kind == "sin":
            dt = wave[1] / 6e8
            out[k] = np.sin(2 * np.pi * wave[2] * dt * t)
        elif kind == "zero":
            out[k] = 0.0
        else:
            raise ValueError(f"unknown waveform {wave!r}")
    return out


def dft_tables(freq, dt: float, t_start: int, n: int):
    """(cos, sin) float64 arrays [n][nf] of 2*pi*freq*dt*t, t = t_start..t_start+n-1."""
    freq = np.asarray(freq, dtype=np.float64).reshape(-1)
    cs = np.zeros((n, freq.size))
    sn = np.zeros((n, freq.size))
    for k in range(n):
        arg = 2 * np.pi * freq * dt * (t_start + k)
        cs[k] = np.cos(arg)
        sn[k] = np.sin(arg)
    return cs, sn


def to_device(a: np.ndarray, device="cuda"):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32)).to(device)
