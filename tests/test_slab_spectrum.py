"""The frequency-domain oracle of the lossy 1D update on CPU: a converged FDTD
run (C oracle, float64) reaches its steady-state transmission, the per-cell
wavenumber solves the cell's transfer matrix, and the surrogate's frame
computed from profile features equals the one computed from the layer table."""
import numpy as np
import pytest

from oracle import ccore
from oracle import slab_spectrum as SS

FREQS = np.linspace(100e6, 3e9, 64)
DT = 0.01 / 6e8


def _small_batch(n, seed):
    from simulation_gb300 import batch1d as B1
    return B1.slab_batch(n, seed=seed, ke_range=(500, 2500), thick=(20, 120))


def _run_coeffs(batch, r, dtype=np.float64):
    a, b = batch.layer_off[r], batch.layer_off[r + 1]
    return SS.cell_coeffs(int(batch.ke[r]), batch.layer_start[a:b], batch.layer_end[a:b], batch.epsr[a:b],
                          batch.sigma[a:b], DT, dtype)


def test_wavenumber_solves_the_cell_recursion():
    """exp(-ik) is an eigenvalue of the cell's transfer matrix, trace = 2 cos k."""
    wdt = 2 * np.pi * FREQS * DT
    for er, sg in [(1.0, 0.0), (4.0, 0.0), (9.0, 0.0), (2.5, 0.01), (7.0, 0.05)]:
        ca, cb = SS.layer_coeffs(er, sg, DT)
        k = SS.yee_wavenumber(ca, cb, wdt)
        z, zh, s = np.exp(1j * wdt), np.exp(0.5j * wdt), np.sin(0.5 * wdt)
        g = (z - ca) / (cb * zh)
        trace = (1 + 4j * s * g) + 1
        np.testing.assert_allclose(2 * np.cos(k), trace, rtol=1e-10, atol=1e-12)
        assert np.all(k.imag <= 0) and np.all(k.real >= 0)
        if sg == 0.0:
            # lossless: sin(k/2) = 2 sqrt(eps_r) sin(w dt / 2) (Courant number 0.5)
            np.testing.assert_allclose(np.sin(k.real / 2), 2 * np.sqrt(er) * np.sin(wdt / 2), rtol=1e-12)


def test_converged_fdtd_reaches_steady_state():
    """Soft derivative-of-Gaussian source, 8000 steps: the DFT ratio of the C
    oracle equals the frequency-domain transmission within 3e-3 (floored)."""
    from simulation_gb300 import batch1d as B1
    from simulation_gb300.sources import dft_tables, wave_values
    batch = _small_batch(12, seed=11)
    ns = 8000
    cs, sn = dft_tables(FREQS, DT, 1, ns)
    lca, lcb = B1.layer_coeffs(batch.epsr, batch.sigma)
    spec = ccore.fd1d_batch(ccore.lib64(), np.float64, batch.ke, batch.layer_off, batch.layer_start,
                            batch.layer_end, lca, lcb, batch.src_k, wave_values(("dgauss", 40, 6.0), 1, ns), ns, cs,
                            sn, batch.probe_in, batch.probe_out)
    T = (spec[:, 2] + 1j * spec[:, 3]) / (spec[:, 0] + 1j * spec[:, 1])
    worst = 0.0
    for r in range(batch.nruns):
        ca, cb = _run_coeffs(batch, r)
        Ts = SS.steady_transmission(ca, cb, int(batch.probe_in[r]), int(batch.probe_out[r]), FREQS, DT)
        err = np.linalg.norm(T[r] - Ts) / max(np.linalg.norm(Ts), 1e-3 * 8)
        worst = max(worst, err)
    assert worst <= 3e-3, worst


def test_frame_from_features_matches_layer_table():
    from simulation_gb300 import batch1d as B1
    from simulation_gb300 import surrogate as S
    batch = B1.slab_batch(6, seed=5)
    feat = S.profile_features(batch)
    for r in range(batch.nruns):
        ca, cb = _run_coeffs(batch, r, np.float32)
        P_tab = SS.propagation_factor(ca, cb, int(batch.probe_in[r]), int(batch.probe_out[r]), FREQS, DT)
        P_feat = SS.propagation_from_features(feat[r], FREQS, DT, S.PROBE_IN, S.PROBE_GAP)
        # eps_r passes through a float32 feature: a relative phase error of ~1e-7
        np.testing.assert_allclose(P_feat, P_tab, rtol=2e-3, atol=1e-30)
        ph = np.angle(P_feat / P_tab)
        assert np.abs(ph).max() < 2e-3


def test_features_hold_both_cells_and_the_left_neighbour():
    from simulation_gb300 import batch1d as B1
    from simulation_gb300 import surrogate as S
    batch = B1.slab_batch(3, seed=2)
    feat = S.profile_features(batch)
    for r in range(3):
        er, sg, _ = SS.features_to_cells(feat[r])
        a, b = batch.layer_off[r], batch.layer_off[r + 1]
        for l in range(a, b):
            lo, hi = int(batch.layer_start[l]), int(batch.layer_end[l])
            np.testing.assert_allclose(er[lo:hi], batch.epsr[l], rtol=1e-6)
            np.testing.assert_allclose(sg[lo:hi], batch.sigma[l], rtol=1e-6, atol=1e-12)
        # channel 0 of bin b is cell 2b-1
        np.testing.assert_array_equal(feat[r, 1:, 0], feat[r, :-1, 2])
        assert feat[r, 0, 0] == 0.0


@pytest.mark.parametrize("kind", ["gauss", "dgauss"])
def test_waveforms(kind):
    from simulation_gb300.sources import wave_values
    v = wave_values((kind, 40, 6.0), 1, 200)
    t = np.arange(1, 201)
    u = (t - 40) / 6.0
    ref = np.exp(-0.5 * u * u) if kind == "gauss" else -u * np.exp(-0.5 * u * u)
    np.testing.assert_allclose(v, ref, rtol=1e-15)
    if kind == "dgauss":
        assert abs(v.sum()) < 1e-8  # no DC content (the pulse starts at 6.5 spreads)
