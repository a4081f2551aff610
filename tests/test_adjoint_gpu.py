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


def _stepwise_gradient(pr, with_nbz=False):
    """dJ/dnaz by the reference-granularity entry points: the forward as
    fdtd2d_step_n calls per checkpoint segment, each segment's states
    recomputed with one-step fdtd2d_pass calls, then fdtd2d_adjoint_step
    (two kernels, in place) once per step."""
    import ctypes as C
    from simulation_gb300 import _lib
    lib = _lib.lib()
    s, p = pr.sim, pr.sim._p
    nx, ny, ns, cp = pr.nx, pr.ny, pr.ns, pr.cp
    # iz only with a conducting box (the lossless update otherwise)
    names = tuple(k for k in ("dz", "iz", "hx", "hy", "ihx", "ihy") if getattr(s, k) is not None)
    z = lambda *sh: torch.zeros(sh, dtype=torch.float32, device="cuda")  # noqa: E731

    def fields(buf):
        f = _lib.Fields2D()
        for k, name in enumerate(names):
            setattr(f, name, buf[k].data_ptr())
        return f

    s.reset()
    trace = z(ns)
    p.probe_i, p.probe_j, p.probe_len = pr.probe[0], pr.probe[1], ns
    s._s.probe_ez = trace.data_ptr()
    ncp = -(-ns // cp)
    ckpt = z(ncp, len(names), nx, ny)
    for c in range(ncp):
        for k, name in enumerate(names):
            ckpt[c, k].copy_(getattr(s, name))
        s.step(min(cp, ns - c * cp))
    s._s.probe_ez = None
    seg, adj, tmp, ez = z(cp, len(names), nx, ny), z(len(names), nx, ny), z(nx, ny), z(nx, ny)
    grad = z(pr.box[2], pr.box[3])
    gradn = z(pr.box[2], pr.box[3]) if with_nbz else None
    box = _lib.Box2D(*pr.box)
    st = _lib.stream_ptr()
    for c in reversed(range(ncp)):
        t0, L = c * cp, min(cp, ns - c * cp)
        seg[0].copy_(ckpt[c])
        for k in range(1, L):
            assert lib.fdtd2d_pass(C.byref(p), C.byref(fields(seg[k - 1])), C.byref(fields(seg[k])), ez.data_ptr(),
                                   t0 + k - 1, 1, None, st) == 0
        for t in range(t0 + L, t0, -1):
            assert lib.fdtd2d_adjoint_step(t, C.byref(p), C.byref(fields(seg[t - t0 - 1])), C.byref(fields(adj)),
                                           tmp.data_ptr(), pr.probe[0], pr.probe[1], 2.0, box, grad.data_ptr(),
                                           gradn.data_ptr() if with_nbz else None, st) == 0
    torch.cuda.synchronize()
    if with_nbz:
        return float((trace.double() ** 2).sum()), trace, grad, gradn
    return float((trace.double() ** 2).sum()), trace, grad


@pytest.mark.parametrize("sigma,cp", [(0.0, 16), (0.05, 21), (0.05, 64)])
def test_one_call_adjoint_equals_stepwise(cuda_lib, sigma, cp):
    """fdtd2d_tm_adjoint_forward/_reverse (recording passes, fused reverse
    kernel, overlapped streams) give the probe trace and dJ/dnaz bit for bit
    equal to the step-by-step entry points; J (summed in double on the
    device) agrees to rounding."""
    pr, eps = _small(cp=cp, sigma=sigma)
    pr.use_graphs = False
    pr.set_eps(eps)
    J = pr.forward()
    g = pr.gradient_naz().clone()
    trace = pr.trace.clone()
    J2, trace2, g2 = _stepwise_gradient(pr)
    assert torch.equal(trace, trace2)
    assert abs(J - J2) <= 1e-12 * abs(J2)
    assert torch.equal(g, g2)
    assert float(g.abs().max()) > 0


def test_one_call_adjoint_single_entry(cuda_lib):
    """fdtd2d_tm_adjoint (forward and reverse in one call) equals the split calls."""
    import ctypes as C
    from simulation_gb300 import _lib
    pr, eps = _small(cp=16, sigma=0.05)
    pr.use_graphs = False
    pr.set_eps(eps)
    J = pr.forward()
    g = pr.gradient_naz().clone()
    trace = torch.zeros_like(pr.trace)
    Jd = torch.zeros(1, dtype=torch.float64, device="cuda")
    g1 = torch.zeros_like(g)
    gn = torch.zeros_like(g)
    _lib.call("fdtd2d_tm_adjoint", C.byref(pr.sim._p), C.byref(pr.ap), trace.data_ptr(), Jd.data_ptr(),
              g1.data_ptr(), gn.data_ptr(), pr.ws.data_ptr(), pr.ws.numel(), _lib.stream_ptr())
    torch.cuda.synchronize()
    assert float(Jd.item()) == J
    assert torch.equal(g1, g)
    assert float(gn.abs().max()) > 0  # dJ/dnbz over the lossy box


@pytest.mark.parametrize("nx,ny,box,off,sigma,cp,kind", [
    (100, 132, (32, 32), 20, 0.05, 21, "soft"),   # no dimension a multiple of the 16 x 32 reverse tile
    (72, 100, (16, 16), 15, 0.0, 9, "hard"),      # lossless box, hard source, odd segments
    (144, 96, (32, 32), 10, 0.05, 10, "hard"),    # even segments only: every reverse launch takes two steps
])
def test_two_step_reverse_equals_stepwise(cuda_lib, nx, ny, box, off, sigma, cp, kind):
    """The reverse sweep (two steps per launch, one for an odd segment's first
    step) gives dJ/dnaz and dJ/dnbz bit for bit equal to one two-kernel
    fdtd2d_adjoint_step per step, on grids that are not multiples of the
    reverse tile, with hard and soft sources, lossless and lossy boxes."""
    import ctypes as C
    from simulation_gb300 import _lib
    from simulation_gb300 import adjoint as A
    pr = A.AdjointProblem(nx=nx, ny=ny, npml=8, box=box, src_offset=off, probe_offset=off, ns=220, checkpoint=cp,
                          wave=("gauss", 30, 8.0), src_kind=kind, sigma_box=sigma)
    pr.use_graphs = False
    eps = torch.as_tensor(np.random.default_rng(5).uniform(1, 4, size=box), dtype=torch.float64)
    pr.set_eps(eps)
    pr.forward()
    lossy = sigma > 0
    g = torch.zeros(box, dtype=torch.float32, device="cuda")
    gn = torch.zeros_like(g)
    _lib.call("fdtd2d_tm_adjoint_reverse", C.byref(pr.sim._p), C.byref(pr.ap), g.data_ptr(),
              gn.data_ptr() if lossy else None, pr.ws.data_ptr(), pr.ws.numel(), _lib.stream_ptr())
    torch.cuda.synchronize()
    ref = _stepwise_gradient(pr, with_nbz=lossy)
    assert torch.equal(g, ref[2])
    assert float(g.abs().max()) > 0
    if lossy:
        assert torch.equal(gn, ref[3])
        assert float(gn.abs().max()) > 0
