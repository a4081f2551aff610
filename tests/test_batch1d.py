"""Batched-slab host logic on CPU: the seeded generator, the C++ planner of
the library (host-only entry point) and the C oracle of one run against the
NumPy oracle."""
import numpy as np
import pytest

from oracle import ccore, fd1d


@pytest.fixture(scope="module")
def B():
    from simulation_gb300 import build
    build.build()
    from simulation_gb300 import batch1d
    return batch1d


def test_generator_is_seeded_and_valid(B):
    a = B.slab_batch(256, seed=3)
    b = B.slab_batch(256, seed=3)
    np.testing.assert_array_equal(a.ke, b.ke)
    np.testing.assert_array_equal(a.layer_start, b.layer_start)
    assert a.ke.min() >= 500 and a.ke.max() <= 20000
    nl = np.diff(a.layer_off)
    assert nl.min() >= 1 and nl.max() <= 8
    th = a.layer_end - a.layer_start
    assert th.min() >= 20 and th.max() <= 400
    assert np.all(a.probe_out + 20 <= a.ke) and np.all(a.probe_in < 40) and np.all(a.probe_in > a.src_k)
    assert a.epsr.min() >= 1 and a.epsr.max() <= 9 and a.sigma.min() >= 0 and a.sigma.max() <= 0.05


@pytest.mark.parametrize("cpt,block", [(8, 1024), (16, 1024), (24, 512), (40, 512), (40, 256)])
def test_planner_places_every_run_once(B, cpt, block):
    ke = np.random.default_rng(1).integers(40, 5000, size=777)
    ke = ke[ke <= cpt * block]
    pl = B.plan(ke, cpt, block)
    nb = int(pl[0])
    assert pl[1] == cpt and pl[2] == block
    bstart = pl[4:4 + nb + 1]
    ent = pl[4 + nb + 1:].reshape(-1, 4)
    assert bstart[0] == 0 and bstart[-1] == ke.size
    np.testing.assert_array_equal(np.sort(ent[:, 0]), np.arange(ke.size))
    for b in range(nb):
        e = ent[bstart[b]:bstart[b + 1]]
        team = ((-(-ke[e[:, 0]] // cpt)) + 31) // 32 * 32
        np.testing.assert_array_equal(e[:, 1], team)
        assert e[:, 1].sum() <= block
        np.testing.assert_array_equal(e[:, 2], np.concatenate([[0], np.cumsum(e[:, 1])[:-1]]))
        multi = e[:, 1] > 32
        assert multi.sum() <= 15
        assert np.all(e[multi, 3] >= 1) and np.all(e[~multi, 3] == 0)
        assert len(set(e[multi, 3])) == multi.sum()


def test_planner_rejects_oversized_runs(B):
    from simulation_gb300 import _lib
    with pytest.raises(_lib.FdtdError):
        B.plan(np.array([100, 9000]), 8, 1024)


def test_c_oracle_batch_equals_numpy_runs(B):
    """oracle_fd1d_batch (the CPU baseline/oracle of the batch) against the
    NumPy oracle run by run."""
    b = B.slab_batch(3, seed=5, ke_range=(500, 900))
    freqs = np.linspace(100e6, 3e9, 8)
    ns = 300
    tab = np.array([fd1d.gaussian(t, 50, 10.0) for t in range(1, ns + 1)])
    dc = np.array([fd1d.dft_phase(t, freqs, B.DT)[0] for t in range(1, ns + 1)])
    ds = np.array([fd1d.dft_phase(t, freqs, B.DT)[1] for t in range(1, ns + 1)])
    lca, lcb = B.layer_coeffs(b.epsr, b.sigma)
    spec = ccore.fd1d_batch(ccore.lib64(), np.float64, b.ke, b.layer_off, b.layer_start, b.layer_end, lca, lcb,
                            b.src_k, tab, ns, dc, ds, b.probe_in, b.probe_out)
    for r in range(3):
        ca, cb = b.coefficients(r)
        st = fd1d.run(int(b.ke[r]), ns, "cacb", ca=ca, cb=cb, src_kind="soft", src_k=b.src_k,
                      wave=("gauss", 50, 10.0), freq=freqs, dt=B.DT, probes=(int(b.probe_in[r]), int(b.probe_out[r])))
        np.testing.assert_array_equal(spec[r, 0], st.r_pr[0])
        np.testing.assert_array_equal(spec[r, 1], st.i_pr[0])
        np.testing.assert_array_equal(spec[r, 2], st.r_pr[1])
        np.testing.assert_array_equal(spec[r, 3], st.i_pr[1])
