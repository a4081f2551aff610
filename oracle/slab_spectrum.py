"""Frequency-domain restatement of the lossy 1D update (oracle only).

Test infrastructure: checks the batched FDTD spectra and the surrogate's
propagation frame; nothing in the library imports it.

The lossy 1D program of fd1d/program/fd1d_1_5.py (coefficients :37-44,
E update :65, H update :72) is, for one frequency w and z = exp(i w dt),
the linear recursion

    E_k (z - ca_k) = cb_k z^1/2 (H_{k-1} - H_k)          (E update)
    H_k (z^1/2 - z^-1/2) = 0.5 (E_k - E_{k+1})            (H update)

with the state (E_k, H_{k-1}) carried cell to cell by a 2x2 matrix of
determinant 1.  ``steady_transmission`` walks it from a purely outgoing wave
behind the exit probe back to the entry probe: the ratio E_out/E_in is the
infinite-time transmission that a converged FDTD run's DFT ratio approaches.
``yee_wavenumber`` is the plane-wave solution of one uniform cell,
sin^2(k/2) = (z^1/2 - ca z^-1/2) sin(w dt/2) / (i cb).
"""
from __future__ import annotations

import numpy as np

EPS0 = 8.854e-12  # fd1d/program/fd1d_1_5.py:40


def layer_coeffs(epsr, sigma, dt):
    """(ca, cb) float64, fd1d/program/fd1d_1_5.py:41-43."""
    epsr = np.asarray(epsr, dtype=np.float64)
    epsf = dt * np.asarray(sigma, dtype=np.float64) / (2 * EPS0 * epsr)
    return (1 - epsf) / (1 + epsf), 0.5 / (epsr * (1 + epsf))


def yee_wavenumber(ca, cb, wdt):
    """Complex wavenumber per cell of the wave travelling to +x (Re k > 0; it
    decays, Im k <= 0, in a passive cell)."""
    ca, cb, wdt = np.broadcast_arrays(np.asarray(ca, float), np.asarray(cb, float), np.asarray(wdt, float))
    s, c = np.sin(0.5 * wdt), np.cos(0.5 * wdt)
    Q = (c * (1 - ca) + 1j * s * (1 + ca)) * s / (1j * cb)
    k = 2 * np.arcsin(np.sqrt(Q + 0j))
    flip = (k.real < 0) | ((k.real == 0) & (k.imag > 0))
    return np.where(flip, -k, k)


def cell_coeffs(ke, starts, ends, epsr, sigma, dt, ca_dtype=np.float32):
    """Per-cell (ca, cb) of one run (vacuum 1, 0.5), rounded like the device copies."""
    ca = np.ones(ke)
    cb = np.full(ke, 0.5)
    lca, lcb = layer_coeffs(epsr, sigma, dt)
    for a, b, x, y in zip(starts, ends, lca, lcb):
        ca[a:b] = x
        cb[a:b] = y
    return ca.astype(ca_dtype).astype(np.float64), cb.astype(ca_dtype).astype(np.float64)


def steady_transmission(ca, cb, probe_in, probe_out, freqs, dt):
    """E(probe_out)/E(probe_in) of the steady state driven from the left, with
    only an outgoing (vacuum) wave at and beyond probe_out."""
    wdt = 2 * np.pi * np.asarray(freqs, dtype=np.float64) * dt
    z = np.exp(1j * wdt)
    zh = np.exp(0.5j * wdt)
    s = np.sin(0.5 * wdt)
    lam = np.exp(-1j * yee_wavenumber(1.0, 0.5, wdt))
    E = np.ones_like(z)
    H = 0.5 * (1 / lam - 1) / (2j * s)  # H_{probe_out-1} of the outgoing wave
    for k in range(probe_out - 1, probe_in - 1, -1):
        g = (z - ca[k]) / (cb[k] * zh)
        E, H = E + 4j * s * H, g * E + (1 + 4j * s * g) * H
    return 1.0 / E


def propagation_factor(ca, cb, probe_in, probe_out, freqs, dt):
    """exp(-i sum_k k_cell) over cells probe_in .. probe_out-1."""
    wdt = 2 * np.pi * np.asarray(freqs, dtype=np.float64) * dt
    K = np.zeros(wdt.shape, dtype=np.complex128)
    for k in range(probe_in, probe_out):
        K += yee_wavenumber(ca[k], cb[k], wdt)
    return np.exp(-1j * K)


def features_to_cells(feat, eps_scale=8.0, sig_scale=0.05):
    """(eps_r, sigma) per cell from [nbins][6] features (cells 2b-1, 2b, 2b+1)."""
    nb = feat.shape[0]
    e = np.empty(2 * nb)
    s = np.empty(2 * nb)
    e[0::2], e[1::2] = feat[:, 1], feat[:, 2]
    s[0::2], s[1::2] = feat[:, 4], feat[:, 5]
    return 1.0 + eps_scale * e.astype(np.float64), sig_scale * s.astype(np.float64), (e != 0) | (s != 0)


def propagation_from_features(feat, freqs, dt, probe_in, probe_gap, eps_scale=8.0, sig_scale=0.05):
    """The surrogate's frame for one profile, from its features alone (as the kernel does)."""
    er, sg, solid = features_to_cells(feat, eps_scale, sig_scale)
    last = int(np.nonzero(solid)[0].max()) if solid.any() else -1
    pout = max(last + 1, probe_in) + probe_gap
    n = max(pout, er.size)
    ca = np.ones(n)
    cb = np.full(n, 0.5)
    eaf = dt * sg / (2 * EPS0 * er)
    ca[:er.size] = ((1 - eaf) / (1 + eaf)).astype(np.float32)
    cb[:er.size] = (0.5 / (er * (1 + eaf))).astype(np.float32)
    return propagation_factor(ca, cb, probe_in, pout, freqs, dt)
