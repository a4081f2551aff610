"""Plain FP64 torch version of the lossy 2D TM update with PML (oracle only).

Differentiable restatement of fd2d/python/fd2d_3_2.py:62-88 with the lossy E
update of fd2d/python/fd2d_3_4.py:131-136 and a point source after the D
update, written with out-of-place tensor ops so torch.autograd can
differentiate J = sum_t Ez_t(probe)^2 with respect to eps_r on a design box.
Used by the tests to check the GPU adjoint kernel (float64 autograd) and to
evaluate central finite differences.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

from . import fd1d as O1
from . import fd2d as O2

EPS0 = 8.854e-12
DT = 0.01 / 6e8


def objective(eps_box: torch.Tensor, *, nx: int, ny: int, npml: int, box, src, probe, ns: int, wave,
              src_kind: str = "soft", sigma_box: float = 0.0, grade: float = 0.33) -> torch.Tensor:
    dev = eps_box.device
    f64 = dict(dtype=torch.float64, device=dev)
    pml = O2.pmlparam(nx, ny, npml, grade)
    P = {k: torch.as_tensor(getattr(pml, k), **f64) for k in
         ("fx1", "fx2", "fx3", "fy1", "fy2", "fy3", "gx2", "gx3", "gy2", "gy3")}
    i0, j0, bi, bj = box
    nb = sigma_box * DT / EPS0
    naz_box = 1.0 / (eps_box.reshape(bi, bj) + nb)
    naz = F.pad(naz_box, (j0, ny - j0 - bj, i0, nx - i0 - bi), value=1.0)
    nbz = torch.zeros((nx, ny), **f64)
    nbz[i0:i0 + bi, j0:j0 + bj] = nb
    table = torch.as_tensor([O1.source_value(t, wave) for t in range(1, ns + 1)], **f64)
    dz = torch.zeros((nx, ny), **f64)
    iz, hx, hy, ihx, ihy = (torch.zeros((nx, ny), **f64) for _ in range(5))
    ca = (P["gx3"][1:, None] * P["gy3"][None, 1:])
    cb = (P["gx2"][1:, None] * P["gy2"][None, 1:]) * 0.5
    src_mask = torch.zeros((nx, ny), **f64)
    src_mask[src] = 1.0
    J = torch.zeros((), **f64)
    for t in range(ns):
        curl = hy[1:, 1:] - hy[:-1, 1:] - hx[1:, 1:] + hx[1:, :-1]
        dzi = ca * dz[1:, 1:] + cb * curl
        dzn = torch.cat([dz[:1, :], torch.cat([dz[1:, :1], dzi], dim=1)], dim=0)
        if src_kind == "soft":
            dzn = dzn + src_mask * table[t]
        else:
            dzn = dzn * (1 - src_mask) + src_mask * table[t]
        ez = naz * (dzn - iz)
        iz = iz + nbz * ez
        cx = ez[:-1, :-1] - ez[:-1, 1:]
        cy = ez[:-1, :-1] - ez[1:, :-1]
        ihx_i = ihx[:-1, :-1] + cx
        ihy_i = ihy[:-1, :-1] + cy
        hx_i = P["fy3"][None, :-1] * hx[:-1, :-1] + P["fy2"][None, :-1] * (0.5 * cx + P["fx1"][:-1, None] * ihx_i)
        hy_i = P["fx3"][:-1, None] * hy[:-1, :-1] - P["fx2"][:-1, None] * (0.5 * cy + P["fy1"][None, :-1] * ihy_i)

        def paste(full, inner):
            top = torch.cat([inner, full[:-1, -1:]], dim=1)
            return torch.cat([top, full[-1:, :]], dim=0)

        ihx, ihy, hx, hy = paste(ihx, ihx_i), paste(ihy, ihy_i), paste(hx, hx_i), paste(hy, hy_i)
        dz = dzn
        J = J + ez[probe] ** 2
    return J


def gradient(eps_box, **kw):
    """(J, dJ/deps_box) in float64 by autograd."""
    e = eps_box.detach().to(torch.float64).clone().requires_grad_(True)
    J = objective(e, **kw)
    (g,) = torch.autograd.grad(J, e)
    return float(J), g.detach()


def problem_kwargs(pr) -> dict:
    """Keyword arguments of ``objective`` matching a simulation_gb300.adjoint.AdjointProblem."""
    return dict(nx=pr.nx, ny=pr.ny, npml=pr._npml, box=pr.box, src=pr.src, probe=pr.probe, ns=pr.ns,
                wave=pr._wave, src_kind=pr._src_kind, sigma_box=pr.sigma_box, grade=pr._grade)
