"""Gradient of an FDTD objective with respect to the permittivity of a design
region, by a hand-written reverse-time (adjoint) kernel with checkpointing.

The forward map is the lossy 2D TM update with PML of the reference
(fd2d/python/fd2d_3_2.py:62-88, lossy E of fd2d/python/fd2d_3_4.py:131-136)
with a Gaussian point source; the objective is J = sum_t Ez_t(probe)^2.  The
reference has no derivative; this is the library's extension.

The whole schedule is one C-ABI call each way (``fdtd2d_tm_adjoint_forward``
and ``fdtd2d_tm_adjoint_reverse``, or both in ``fdtd2d_tm_adjoint``): the
forward runs fused passes with a stored state every ``checkpoint`` steps and
records Ez at the probe; the reverse recomputes each segment from its
checkpoint with passes that record every step's state (on a second stream,
one segment ahead) and undoes the steps with one fused reverse kernel each,
accumulating dJ/dnaz on the design box.  dJ/deps_r = -naz^2 * dJ/dnaz since
naz = 1/(eps_r + sigma*dt/eps0).  This module only holds the tensors and the
workspace and calls the library.

``FdtdObjective`` wraps forward + reverse as a torch.autograd.Function.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .fd2d import PointSource, SimTM2D, pmlparam

EPS0 = 8.854e-12
DT = 0.01 / 6e8


class AdjointProblem:
    """Design problem on an nx x ny grid with an npml PML.

    The design box (bi x bj cells) is centred; the source sits ``src_offset``
    cells before the box along i (the first axis) and the probe
    ``probe_offset`` cells after it, both on the centre column.
    """

    def __init__(self, nx: int = 1024, ny: int = 1024, npml: int = 16, box=(256, 256), src_offset: int = 200,
                 probe_offset: int = 200, ns: int = 3000, checkpoint: int = 64, wave=("gauss", 40, 12.0),
                 src_kind: str = "soft", sigma_box: float = 0.0, grade: float = 0.33, device="cuda",
                 use_graphs: bool = True):
        if ny % 4:
            raise ValueError("ny must be a multiple of 4")
        self.nx, self.ny, self.ns, self.cp = nx, ny, ns, checkpoint
        self._npml, self._wave, self._src_kind, self._grade = npml, wave, src_kind, grade
        self.device = torch.device(device)
        bi, bj = box
        self.box = (nx // 2 - bi // 2, ny // 2 - bj // 2, bi, bj)
        i0, j0 = self.box[0], self.box[1]
        self.src = (i0 - src_offset, ny // 2)
        self.probe = (i0 + bi - 1 + probe_offset, ny // 2)
        if not (npml < self.src[0] and self.probe[0] < nx - npml):
            raise ValueError("source/probe inside the PML or outside the grid")
        self.sigma_box = sigma_box
        # a box without conductivity runs the lossless E update: with nbz = 0
        # the lossy one keeps iz = 0, and naz*(dz - 0) = naz*dz exactly, so the
        # values are the same while iz and nbz are neither stored nor read
        self.sim = SimTM2D(nx, ny, pml=pmlparam(nx, ny, npml, grade, device), lossy=sigma_box > 0,
                           source=PointSource(self.src[0], self.src[1], wave, src_kind), ns=ns, device=device,
                           check_finite=True)
        self.trace = torch.zeros(ns, dtype=torch.float32, device=self.device)
        self.J_dev = torch.zeros(1, dtype=torch.float64, device=self.device)
        self.grad_naz = torch.zeros((bi, bj), dtype=torch.float32, device=self.device)
        self.ncp = -(-ns // checkpoint)
        self.ap = _lib.AdjointParams2D(ns, checkpoint, self.probe[0], self.probe[1], 2.0,
                                       _lib.Box2D(*self.box))
        n = _lib.lib().fdtd2d_tm_adjoint_workspace_size(C.byref(self.sim._p), C.byref(self.ap))
        if n == 0:
            raise ValueError("fdtd2d_tm_adjoint_workspace_size rejected the problem")
        self.ws = torch.empty(n, dtype=torch.uint8, device=self.device)
        self.J = None
        # the loops are static for a problem (pointers, steps, segment order):
        # from the second call on, each sweep replays a CUDA graph of itself
        self.use_graphs = use_graphs
        self._graph = {"forward": None, "reverse": None}
        self._warm = {"forward": False, "reverse": False}

    # ------------------------------------------------------------ material
    def set_eps(self, eps_box: torch.Tensor) -> None:
        """naz/nbz from eps_r on the box (float64 formula, fd2d/python/fd2d_3_4.py:192-193)."""
        i0, j0, bi, bj = self.box
        e = eps_box.detach().to(self.device, torch.float64).reshape(bi, bj)
        nb = self.sigma_box * DT / EPS0
        self.sim.naz.fill_(1.0)
        self.sim.naz[i0:i0 + bi, j0:j0 + bj] = (1.0 / (e + nb)).float()
        if self.sim.nbz is not None:
            self.sim.nbz.zero_()
            self.sim.nbz[i0:i0 + bi, j0:j0 + bj] = nb

    # ------------------------------------------------------------ forward
    def _run(self, name: str, body) -> None:
        """body() eagerly on the first call; later calls capture it once into a
        CUDA graph and replay that (same kernels, same arguments)."""
        if not self.use_graphs or not self._warm[name]:
            body()
            self._warm[name] = True
            return
        g = self._graph[name]
        if g is None:
            g = torch.cuda.CUDAGraph()
            cap = torch.cuda.Stream(device=self.device)
            cap.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(cap):
                with torch.cuda.graph(g, stream=cap):
                    body()
            torch.cuda.current_stream(self.device).wait_stream(cap)
            self._graph[name] = g
        g.replay()

    def forward(self) -> float:
        """Run the time loop with checkpoints; returns J = sum_t Ez_t(probe)^2."""
        def body():
            _lib.call("fdtd2d_tm_adjoint_forward", C.byref(self.sim._p), C.byref(self.ap), self.trace.data_ptr(),
                      self.J_dev.data_ptr(), self.ws.data_ptr(), self.ws.numel(), _lib.stream_ptr())

        self._run("forward", body)
        self.sim.t = self.ns
        self.J = float(self.J_dev.item())
        return self.J

    # ------------------------------------------------------------ reverse
    def gradient_naz(self) -> torch.Tensor:
        """dJ/dnaz on the design box (float32 [bi][bj]) by the reverse sweep
        over the checkpoints of the last ``forward``."""
        def body():
            _lib.call("fdtd2d_tm_adjoint_reverse", C.byref(self.sim._p), C.byref(self.ap),
                      self.grad_naz.data_ptr(), None, self.ws.data_ptr(), self.ws.numel(), _lib.stream_ptr())

        self._run("reverse", body)
        return self.grad_naz

    def gradient_eps(self) -> torch.Tensor:
        """dJ/deps_r on the design box (float64): -naz^2 * dJ/dnaz."""
        g = self.gradient_naz().double()
        i0, j0, bi, bj = self.box
        naz = self.sim.naz[i0:i0 + bi, j0:j0 + bj].double()
        return -naz * naz * g


class FdtdObjective(torch.autograd.Function):
    """J(eps_r) = sum_t Ez_t(probe)^2 with its gradient from the adjoint kernel."""

    @staticmethod
    def forward(ctx, eps_box, problem: AdjointProblem):
        problem.set_eps(eps_box)
        J = problem.forward()
        ctx.problem = problem
        ctx.shape = eps_box.shape
        return torch.tensor(J, dtype=torch.float64, device=eps_box.device)

    @staticmethod
    def backward(ctx, gJ):
        g = ctx.problem.gradient_eps().to(gJ.device).reshape(ctx.shape)
        return gJ * g, None


def design_problem(seed: int = 0, device="cuda", **kw):
    """The 1024^2 adjoint benchmark: 16-cell PML, 256^2 centred design box with
    eps_r ~ U[1, 4] (seeded), source 200 cells before and probe 200 cells after
    the box, 3000 steps, checkpoints every 64 steps.  Returns (problem, eps)."""
    pr = AdjointProblem(device=device, **kw)
    rng = np.random.default_rng(seed)
    bi, bj = pr.box[2], pr.box[3]
    eps = torch.as_tensor(rng.uniform(1.0, 4.0, size=(bi, bj)), dtype=torch.float64)
    return pr, eps
