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
    """params: name -> float64 tensor; inp [B][N][cin] float64 -> out [B][D]."""
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


def apply_frame(frame: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
    """T = P (.) y for spectra stored [Re | Im]."""
    nf = y.shape[1] // 2
    pr, pi, yr, yi = frame[:, :nf], frame[:, nf:], y[:, :nf], y[:, nf:]
    return torch.cat([pr * yr - pi * yi, pr * yi + pi * yr], dim=1)


def loss_and_grads(params: dict, inp: torch.Tensor, target: torch.Tensor, layers: int, modes: int,
                   frame: torch.Tensor | None = None, rel_floor2: float | None = None):
    """Loss, network output and parameter gradients.  ``frame``: loss on
    P (.) y; ``rel_floor2``: per-sample ||o-t||^2 / max(||t||^2, floor2)
    averaged over the batch, else the plain mean squared error."""
    p = {k: v.detach().double().cpu().clone().requires_grad_(True) for k, v in params.items()}
    o = forward(p, inp.double().cpu(), layers, modes)
    out = o if frame is None else apply_frame(frame.double().cpu(), o)
    t = target.double().cpu()
    if rel_floor2 is None:
        loss = ((out - t) ** 2).mean()
    else:
        w = 1.0 / torch.clamp((t ** 2).sum(1), min=rel_floor2)
        loss = (w * ((out - t) ** 2).sum(1)).mean()
    grads = torch.autograd.grad(loss, list(p.values()))
    return float(loss), o.detach(), {k: g for k, g in zip(p.keys(), grads)}
