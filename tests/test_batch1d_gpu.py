"""Batched-slab parity on the GPU: sampled runs against the float64 C oracle,
bitwise independence from the tuning (cells per thread, block size, groups),
and the clock budget that stops a persistent launch without hanging."""
import numpy as np
import pytest
import torch

from oracle import ccore
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _oracle_spec(B, runner, runs, ns):
    b = runner.batch.subset(runs)
    lca, lcb = B.layer_coeffs(b.epsr, b.sigma)
    lca, lcb = lca.astype(np.float32).astype(np.float64), lcb.astype(np.float32).astype(np.float64)
    tab = runner.src_table.double().cpu().numpy()[:ns]
    dc = runner.dft_cos.double().cpu().numpy()[:ns]
    ds = runner.dft_sin.double().cpu().numpy()[:ns]
    return ccore.fd1d_batch(ccore.lib64(), np.float64, b.ke, b.layer_off, b.layer_start, b.layer_end, lca, lcb,
                            b.src_k, tab, ns, dc, ds, b.probe_in, b.probe_out)


def test_sampled_runs_vs_oracle(cuda_lib):
    from simulation_gb300 import batch1d as B
    batch = B.slab_batch(512, seed=7)
    ns = 2000
    runner = B.BatchRunner(batch, nsteps=ns)
    runner.run()
    torch.cuda.synchronize()
    assert int(runner.status.item()) == 0
    assert int(runner.done.sum()) == batch.nruns
    sample = np.random.default_rng(0).choice(batch.nruns, size=64, replace=False)
    ref = _oracle_spec(B, runner, sample, ns)
    got = runner.spec.double().cpu().numpy()[sample]
    worst = max(rel_l2(got[k], ref[k]) for k in range(sample.size))
    assert worst <= 1e-5, f"worst per-run spectrum rel-L2 {worst:.3e}"


def test_tuning_does_not_change_results(cuda_lib):
    from simulation_gb300 import batch1d as B
    batch = B.slab_batch(300, seed=11, ke_range=(500, 20000))  # long enough for two-group splits
    outs = []
    tunings = B.candidate_tunings(batch.ke)
    assert any(len(t["groups"]) > 1 for t in tunings)
    for tun in tunings:
        r = B.BatchRunner(batch, nsteps=600, tuning=tun)
        r.run()
        torch.cuda.synchronize()
        outs.append(r.spec.clone())
        # every run of every group is flagged done, whatever the split
        assert int(r.done.sum()) == batch.nruns, tun
    for o in outs[1:]:
        assert torch.equal(o, outs[0])


def test_clock_budget_stops_cleanly(cuda_lib):
    """A tiny per-block clock budget: the launch returns, FDTD_STATUS_TIMEOUT is
    raised and only some runs are marked done (no hang, context stays usable)."""
    from simulation_gb300 import batch1d as B
    batch = B.slab_batch(2000, seed=2)
    r = B.BatchRunner(batch, nsteps=200)
    r.run(max_cycles=1000)
    torch.cuda.synchronize()
    assert int(r.status.item()) & 2
    assert 0 < int(r.done.sum()) < batch.nruns
    r2 = B.BatchRunner(batch.subset(np.arange(20)), nsteps=50)
    r2.run()
    torch.cuda.synchronize()
    assert int(r2.done.sum()) == 20


def test_runs_bitwise_equal_to_per_function_kernels(cuda_lib):
    """Sampled runs of the batch, replayed one at a time through the 1D
    per-function kernels (fdtd1d_efield / fdtd1d_fourier / fdtd1d_hfield: ca/cb
    form, soft source, two-step-back ABC, DFT at the entry and exit probes),
    give the same spectrum accumulators bit for bit (fd1d/program/fd1d_1_5.py
    with the running DFT of fd1d/program/fd1d_2_2.py:65-71)."""
    from simulation_gb300 import batch1d as B
    from simulation_gb300 import fd1d as G
    batch = B.slab_batch(256, seed=11)
    ns = 1500
    runner = B.BatchRunner(batch, nsteps=ns)
    runner.run()
    torch.cuda.synchronize()
    spec = runner.spec.cpu()
    # short, long and mid-length runs (the longest needs the widest team)
    order = np.argsort(batch.ke)
    for r in (int(order[0]), int(order[len(order) // 2]), int(order[-1])):
        nx = int(batch.ke[r])
        ca = np.ones(nx)
        cb = np.full(nx, 0.5)
        for l in range(batch.layer_off[r], batch.layer_off[r + 1]):
            lca, lcb = B.layer_coeffs(batch.epsr[l:l + 1], batch.sigma[l:l + 1])
            ca[batch.layer_start[l]:batch.layer_end[l]] = lca[0]
            cb[batch.layer_start[l]:batch.layer_end[l]] = lcb[0]
        sim = G.Sim1D(nx, "cacb", ca=ca, cb=cb, src_kind="soft", src_k=int(batch.src_k), wave=("gauss", 50, 10.0),
                      freq=runner.freqs, dt=B.DT, probes=(int(batch.probe_in[r]), int(batch.probe_out[r])), ns=ns)
        sim.step_per_function(ns)
        torch.cuda.synchronize()
        got = spec[r]  # [4][nf]: re/im at the entry probe, re/im at the exit probe
        want = torch.stack([sim.r_pr[0], sim.i_pr[0], sim.r_pr[1], sim.i_pr[1]]).cpu()
        assert torch.equal(got, want), f"run {r} (ke={nx}): max {float((got - want).abs().max()):.3e}"
