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
