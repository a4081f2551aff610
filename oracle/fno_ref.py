"""FP64 CPU restatement of the surrogate network (oracle only).

The same 1D Fourier neural operator as simulation_gb300.surrogate, written
with float64 torch ops on the CPU so torch.autograd gives reference gradients
for the GPU's hand-written BF16 forward/backward kernels.
"""
from __future__ import annotations

import numpy as np
import torch


def dft_matrices(n: int, m: int):
    k = np.arange(m)[:, None]
    x = np.arange(n)[None, :]
    th = 2 * np.pi * k * x / n
    phi = np.concatenate([np.cos(th), -np.sin(th)], axis=0)
    a = np.full(m, 2.0 / n)
    a[0] = 1.0 / n
    psi = np.concatenate([(a[:, None] * np.cos(th)).T, (-a[:, None] * np.sin(th)).T], axis=1)
    return torch.as_tensor(phi), torch.as_tensor(psi)


def gelu(z):
    """GELU, tanh form (Hendrycks & Gimpel 2016), as the GPU kernels use it."""
    return 0.5 * z * (1.0 + torch.tanh(np.sqrt(2.0 / np.pi) * (z + 0.044715 * z ** 3)))


def forward(params: dict, inp: torch.Tensor, layers: int, modes: int) -> torch.Tensor:
    """params: name -> float64 tensor; inp [B][N][2] float64 -> out [B][D]."""
    B, N, _ = inp.shape
    phi, psi = dft_matrices(N, modes)
    x = inp @ params["P"].T + params["pb"]                       # [B][N][C]
    for l in range(layers):
        F = torch.einsum("bnc,jn->bcj", x, phi)                   # [B][C][2M]
        Fr, Fi = F[..., :modes], F[..., modes:]                   # [B][C][M]
        Rr, Ri = params[f"L{l}.Rr"], params[f"L{l}.Ri"]           # [M][Co][Ci]
        Gr = torch.einsum("koi,bik->bok", Rr, Fr) - torch.einsum("koi,bik->bok", Ri, Fi)
        Gi = torch.einsum("koi,bik->bok", Ri, Fr) + torch.einsum("koi,bik->bok", Rr, Fi)
        G = torch.cat([Gr, Gi], dim=-1)                           # [B][C][2M]
        y2 = torch.einsum("nj,bcj->bnc", psi, G)
        x = gelu(x @ params[f"L{l}.W"].T + params[f"L{l}.b"] + y2)
    h = x.mean(dim=1)
    a1 = gelu(h @ params["H1"].T + params["hb1"])
    return a1 @ params["H2"].T + params["hb2"]


def loss_and_grads(params: dict, inp: torch.Tensor, target: torch.Tensor, layers: int, modes: int):
    p = {k: v.detach().double().cpu().clone().requires_grad_(True) for k, v in params.items()}
    o = forward(p, inp.double().cpu(), layers, modes)
    loss = ((o - target.double().cpu()) ** 2).mean()
    grads = torch.autograd.grad(loss, list(p.values()))
    return float(loss), o.detach(), {k: g for k, g in zip(p.keys(), grads)}
