"""The neural-operator surrogate on the GPU: forward and gradients of the
hand-written BF16 kernels against the FP64 CPU oracle, training that lowers
the loss, and the FDTD judge/fallback."""
import numpy as np
import pytest
import torch

from oracle import fno_ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _small_model():
    from simulation_gb300 import surrogate as S
    return S.FNO(seed=1, nbins=256, width=128, modes=16, layers=2, hidden=256, out=128)


def test_forward_and_gradients_vs_fp64_oracle(cuda_lib):
    m = _small_model()
    g = torch.Generator().manual_seed(0)
    # the output layer starts at zero; give it values so every gradient is exercised
    m.p["H2"].copy_(((torch.rand(m.p["H2"].shape, generator=g) * 2 - 1) / 16).cuda())
    m.p["hb2"].copy_(((torch.rand(m.p["hb2"].shape, generator=g) * 2 - 1) / 10).cuda())
    m._refresh_bf16()
    inp = torch.rand((8, 256, 2), generator=g)
    tgt = torch.randn((8, 128), generator=g) * 0.3
    loss = m.loss_and_grad(inp.cuda(), tgt.cuda())
    o_gpu = m._saved  # noqa: F841  (kept alive until here)
    torch.cuda.synchronize()
    params = {k: v.detach().cpu() for k, v in m.p.items()}
    l_ref, o_ref, g_ref = fno_ref.loss_and_grads(params, inp, tgt, layers=2, modes=16)
    o = m.forward(inp.cuda()).cpu().double()
    assert rel_l2(o.numpy(), o_ref.numpy()) <= 3e-2
    assert abs(float(loss.item()) - l_ref) <= 3e-2 * l_ref
    worst = {}
    for k, gr in g_ref.items():
        worst[k] = rel_l2(m.g[k].cpu().double().numpy(), gr.numpy())
    bad = {k: v for k, v in worst.items() if v > 6e-2}
    assert not bad, f"gradient rel-L2 above 6e-2: {bad}"


def test_training_lowers_loss(cuda_lib):
    m = _small_model()
    g = torch.Generator().manual_seed(2)
    X = torch.rand((64, 256, 2), generator=g).cuda()
    W = torch.randn((2, 128), generator=g).cuda()
    Y = torch.tanh(X.mean(1) @ W).contiguous()  # a smooth function of the profile
    first = float(m.loss_and_grad(X, Y).item())
    for _ in range(60):
        m.loss_and_grad(X, Y)
        m.adam_step(1e-3)
    last = float(m.loss_and_grad(X, Y).item())
    assert last < 0.5 * first, (first, last)


def test_judge_replaces_bad_predictions(cuda_lib):
    """Every spot-checked profile ends within the tolerance: either the network
    was already that close, or its FDTD spectrum replaced the prediction."""
    from simulation_gb300 import batch1d as B1
    from simulation_gb300 import surrogate as S
    m = S.FNO(seed=0)
    m.p["hb2"].fill_(0.05)  # a deliberately wrong network
    m._refresh_bf16()
    batch = B1.slab_batch(200, seed=4)
    judge = S.JudgedSurrogate(m, check_frac=0.05, tol=0.01, nsteps=2000, seed=0)
    pred, info = judge(batch)
    assert info["checked"] == 10 and info["fell_back"] == 10
    r = B1.BatchRunner(batch.subset(info["checked_idx"]), nsteps=2000)
    r.run()
    ref = S.spectrum_targets(r.transmission())
    assert np.all(S.rel_l2_spectrum(pred[info["checked_idx"]], ref) <= 0.01)
