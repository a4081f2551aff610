"""Gradient of an FDTD objective with respect to the permittivity of a design
region, by a hand-written reverse-time (adjoint) kernel with checkpointing.

The forward map is the lossy 2D TM update with PML of the reference
(fd2d/python/fd2d_3_2.py:62-88, lossy E of fd2d/python/fd2d_3_4.py:131-136)
with a Gaussian point source; the objective is J = sum_t Ez_t(probe)^2.  The
reference has no derivative; this is the library's extension.

Forward: the fused kernel (``fdtd2d_step_n``) runs the time loop, records
Ez at the probe every step and copies the fields to a checkpoint every
``checkpoint`` steps.  Reverse: for each segment, last first, the states of
the segment are recomputed from its checkpoint (``fdtd2d_pass``, one step per
pass, bitwise equal to the forward; on a second stream, one segment ahead of
the sweep), then ``fdtd2d_adjoint_step`` walks the segment backwards
accumulating dJ/dnaz on the design box;
dJ/deps_r = -naz^2 * dJ/dnaz since naz = 1/(eps_r + sigma*dt/eps0).

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
        self.sim = SimTM2D(nx, ny, pml=pmlparam(nx, ny, npml, grade, device), lossy=True,
                           source=PointSource(self.src[0], self.src[1], wave, src_kind), ns=ns, device=device,
                           check_finite=True)
        self.trace = torch.zeros(ns, dtype=torch.float32, device=self.device)
        self.sim._p.probe_i, self.sim._p.probe_j, self.sim._p.probe_len = self.probe[0], self.probe[1], ns
        self.sim._s.probe_ez = self.trace.data_ptr()
        self.ncp = -(-ns // checkpoint)
        z = lambda *s: torch.zeros(s, dtype=torch.float32, device=self.device)  # noqa: E731
        self.ckpt = z(self.ncp, 6, nx, ny)
        self.seg = z(2, checkpoint, 6, nx, ny)  # two segments: one recomputed while the other is swept
        self.adj = z(6, nx, ny)
        self.tmp = z(nx, ny)
        self.ez_scratch = z(nx, ny)
        self.grad_naz = z(bi, bj)
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
        self.sim.nbz.zero_()
        self.sim.naz[i0:i0 + bi, j0:j0 + bj] = (1.0 / (e + nb)).float()
        self.sim.nbz[i0:i0 + bi, j0:j0 + bj] = nb

    FIELDS = ("dz", "iz", "hx", "hy", "ihx", "ihy")

    def _fields(self, buf) -> _lib.Fields2D:
        f = _lib.Fields2D()
        for k, name in enumerate(self.FIELDS):
            setattr(f, name, buf[k].data_ptr())
        return f

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
        s = self.sim

        def body():
            s.reset()
            self.trace.zero_()
            for c in range(self.ncp):
                for k, name in enumerate(self.FIELDS):
                    self.ckpt[c, k].copy_(getattr(s, name))
                s.step(min(self.cp, self.ns - c * self.cp))

        self._run("forward", body)
        s.t = self.ns
        self.J = float((self.trace.double() ** 2).sum())
        return self.J

    # ------------------------------------------------------------ reverse
    def gradient_naz(self) -> torch.Tensor:
        """dJ/dnaz on the design box (float32 [bi][bj]) by the reverse sweep.

        Segments are swept last first.  While the current stream walks segment
        c backwards, a second stream recomputes the states of segment c-1 into
        the other half of ``seg``; events order each buffer's reuse.  The work
        per kernel is unchanged, so the gradient is the same bit for bit."""
        if not hasattr(self, "_side"):
            self._side = torch.cuda.Stream(device=self.device)
        self._run("reverse", self._reverse)
        return self.grad_naz

    def _reverse(self) -> None:
        lib = _lib.lib()
        main = torch.cuda.current_stream(self.device)
        side = self._side
        st_main, st_side = main.cuda_stream, side.cuda_stream
        p = self.sim._p
        self.adj.zero_()
        self.grad_naz.zero_()
        adj = self._fields(self.adj)
        i0, j0, bi, bj = self.box
        box = _lib.Box2D(i0, j0, bi, bj)
        seg_f = [[self._fields(self.seg[b, k]) for k in range(self.cp)] for b in range(2)]
        ready = [torch.cuda.Event(), torch.cuda.Event()]  # buffer b holds its segment's states
        free = [torch.cuda.Event(), torch.cuda.Event()]   # the sweep over buffer b has finished
        side.wait_stream(main)  # the forward's checkpoints and the zeroing above come first

        def recompute(c: int, b: int) -> list:
            t_start = c * self.cp
            L = min(self.cp, self.ns - t_start)
            states = [self._fields(self.ckpt[c])] + seg_f[b][1:L]
            for k in range(1, L):
                rc = lib.fdtd2d_pass(C.byref(p), C.byref(states[k - 1]), C.byref(states[k]),
                                     self.ez_scratch.data_ptr(), t_start + k - 1, 1, None, st_side)
                if rc:
                    raise _lib.FdtdError(rc, "fdtd2d_pass")
            ready[b].record(side)
            return states

        order = list(reversed(range(self.ncp)))
        states_of = {order[0]: recompute(order[0], 0)}
        for idx, c in enumerate(order):
            b = idx % 2
            if idx + 1 < len(order):
                nb = 1 - b
                if idx >= 1:
                    side.wait_event(free[nb])  # the sweep of the segment before used buffer nb
                states_of[order[idx + 1]] = recompute(order[idx + 1], nb)
            main.wait_event(ready[b])
            states = states_of.pop(c)
            t_start = c * self.cp
            L = min(self.cp, self.ns - t_start)
            for t in range(t_start + L, t_start, -1):
                rc = lib.fdtd2d_adjoint_step(t, C.byref(p), C.byref(states[t - t_start - 1]), C.byref(adj),
                                             self.tmp.data_ptr(), self.probe[0], self.probe[1], 2.0, box,
                                             self.grad_naz.data_ptr(), None, st_main)
                if rc:
                    raise _lib.FdtdError(rc, "fdtd2d_adjoint_step")
            free[b].record(main)

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
