"""Adjoint gradient on the GPU (FP32 reverse kernel with checkpoints) against
autograd through the plain FP64 torch version of the same update, against
central finite differences, and independent of the checkpoint interval."""
import numpy as np
import pytest
import torch

from oracle import torch_fd2d as T
from tests.conftest import assert_parity

pytestmark = pytest.mark.gpu


def _small(cp=16, ns=300, sigma=0.0):
    from simulation_gb300 import adjoint as A
    pr = A.AdjointProblem(nx=128, ny=128, npml=8, box=(32, 32), src_offset=30, probe_offset=30, ns=ns,
                          checkpoint=cp, wave=("gauss", 40, 12.0), sigma_box=sigma)
    eps = torch.as_tensor(np.random.default_rng(3).uniform(1, 4, size=(32, 32)), dtype=torch.float64)
    return pr, eps


@pytest.mark.parametrize("sigma", [0.0, 0.05])
def test_adjoint_vs_fp64_autograd_128(cuda_lib, sigma):
    from simulation_gb300 import adjoint as A
    pr, eps = _small(sigma=sigma)
    e = eps.clone().requires_grad_(True)
    J = A.FdtdObjective.apply(e, pr)
    J.backward()
    g_gpu = e.grad.detach().cpu().numpy()
    Jr, g_ref = T.gradient(eps.cuda(), **T.problem_kwargs(pr))
    assert abs(float(J) - Jr) <= 1e-4 * abs(Jr)
    assert_parity(g_gpu, g_ref.cpu().numpy(), tol=1e-4, what="dJ/deps")


def test_checkpoint_interval_does_not_change_gradient(cuda_lib):
    a, eps = _small(cp=16)
    b, _ = _small(cp=64)
    a.set_eps(eps)
    b.set_eps(eps)
    a.forward()
    b.forward()
    assert a.J == b.J
    assert torch.equal(a.gradient_naz(), b.gradient_naz())


def test_graph_replay_equals_eager(cuda_lib):
    """From the second call on, forward and reverse replay captured CUDA
    graphs: J and the gradient equal the eager sweeps bit for bit, also after
    the permittivity changes (the graphs read naz/nbz in place)."""
    a, eps = _small(cp=16)
    b, _ = _small(cp=16)
    b.use_graphs = False
    a.set_eps(eps)
    b.set_eps(eps)
    for _ in range(3):  # eager, capture + replay, replay
        ja = a.forward()
        ga = a.gradient_naz().clone()
    assert a._graph["forward"] is not None and a._graph["reverse"] is not None
    jb = b.forward()
    gb = b.gradient_naz().clone()
    assert ja == jb
    assert torch.equal(ga, gb)
    eps2 = eps * 1.1
    a.set_eps(eps2)
    b.set_eps(eps2)
    assert a.forward() == b.forward()
    assert torch.equal(a.gradient_naz(), b.gradient_naz())


def test_adjoint_vs_central_fd_config4(cuda_lib):
    """1024^2, 16-cell PML, 256^2 design box, 3000 steps, checkpoints every 64:
    the reverse kernel's dJ/deps on 32 random cells vs central differences with
    h = 1e-3 (evaluated by the FP64 forward)."""
    from simulation_gb300 import adjoint as A
    pr, eps = A.design_problem(seed=0)
    pr.set_eps(eps)
    J = pr.forward()
    g = pr.gradient_eps().cpu().numpy()
    kw = T.problem_kwargs(pr)
    rng = np.random.default_rng(1)
    cells = [(int(a), int(b)) for a, b in zip(rng.integers(0, 256, 32), rng.integers(0, 256, 32))]
    h = 1e-3
    e64 = eps.cuda()
    with torch.no_grad():
        J0 = float(T.objective(e64, **kw))
        assert abs(J - J0) <= 1e-4 * abs(J0)
        errs = []
        for (a, b) in cells:
            ep, em = e64.clone(), e64.clone()
            ep[a, b] += h
            em[a, b] -= h
            fd = (float(T.objective(ep, **kw)) - float(T.objective(em, **kw))) / (2 * h)
            errs.append((abs(fd - g[a, b]), abs(fd)))
    err = np.array([e for e, _ in errs])
    ref = np.array([d for _, d in errs])
    rl2 = float(np.linalg.norm(err) / np.linalg.norm(ref))
    print(f"central FD vs adjoint on 32 cells: rel-L2 {rl2:.3e}, worst {err.max():.3e} of max |fd| {ref.max():.3e}")
    assert rl2 <= 1e-3, f"rel-L2 {rl2:.3e}"
