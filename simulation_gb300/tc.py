"""Torch-facing wrapper of the library's BF16 tensor-core GEMM (``fdtd_gemm_bf16``).

``gemm`` computes ``C = epilogue(alpha * A @ B')`` where B' is ``B.T`` for a
K-major B ([N][K]) and ``B`` for an MN-major B ([K][N]); A may be given as
[M][K] or, with ``a_mn=True``, as its transpose [K][M] (no copy is made).  All
operands are BF16 CUDA tensors; the accumulator is FP32 in tensor memory.
Batched operands are 3-D tensors with the batch first (stride 0 = shared).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib


def _ld_stride(t: torch.Tensor):
    if t.dim() == 2:
        return t.stride(0), 0, 1
    return t.stride(1), t.stride(0), t.shape[0]


def gemm(A: torch.Tensor, B: torch.Tensor, *, a_mn: bool = False, b_mn: bool = False, out: torch.Tensor | None = None,
         out_dtype=torch.float32, bias: torch.Tensor | None = None, residual: torch.Tensor | None = None,
         alpha: float = 1.0, gelu: bool = False, accumulate: bool = False, pre: torch.Tensor | None = None,
         status: torch.Tensor | None = None, mn_lbo: int = 0, mn_sbo: int = 0, second=None) -> torch.Tensor:
    """``second`` = (A2, B2, a2_mn, b2_mn) adds A2 @ B2' to the accumulator before
    the epilogue (same output shape)."""
    for t in (A, B):
        if t.dtype != torch.bfloat16 or not t.is_cuda:
            raise TypeError("A and B must be BF16 CUDA tensors")
        if t.stride(-1) != 1:
            raise ValueError("innermost dimension must be contiguous")
    batch = max(A.shape[0] if A.dim() == 3 else 1, B.shape[0] if B.dim() == 3 else 1)
    M = A.shape[-1] if a_mn else A.shape[-2]
    K = A.shape[-2] if a_mn else A.shape[-1]
    N = B.shape[-1] if b_mn else B.shape[-2]
    Kb = B.shape[-2] if b_mn else B.shape[-1]
    if K != Kb:
        raise ValueError(f"inner dimensions differ: {K} vs {Kb}")
    shape = (batch, M, N) if (A.dim() == 3 or B.dim() == 3) else (M, N)
    if out is None:
        out = torch.empty(shape, dtype=out_dtype, device=A.device)
    d = _lib.GemmDesc()
    d.M, d.N, d.K, d.batch = M, N, K, batch
    lda, sa, _ = _ld_stride(A)
    ldb, sb, _ = _ld_stride(B)
    d.A, d.lda, d.stride_a, d.a_mn_major = A.data_ptr(), lda, sa, int(a_mn)
    d.B, d.ldb, d.stride_b, d.b_mn_major = B.data_ptr(), ldb, sb, int(b_mn)
    ldc, sc, _ = _ld_stride(out)
    if out.dtype == torch.float32:
        d.C32 = out.data_ptr()
    elif out.dtype == torch.bfloat16:
        d.C16 = out.data_ptr()
    else:
        raise TypeError("output must be float32 or bfloat16")
    d.ldc, d.stride_c = ldc, sc
    if bias is not None:
        d.bias = bias.data_ptr()
    if residual is not None:
        ldr, sr, _ = _ld_stride(residual)
        d.res16, d.ldr, d.stride_r = residual.data_ptr(), ldr, sr
    if pre is not None:
        d.pre16 = pre.data_ptr()
    d.alpha, d.act, d.accumulate = float(alpha), int(gelu), int(accumulate)
    d.mn_lbo, d.mn_sbo = mn_lbo, mn_sbo
    if second is not None:
        A2, B2, a2_mn, b2_mn = second
        K2 = A2.shape[-2] if a2_mn else A2.shape[-1]
        K2b = B2.shape[-2] if b2_mn else B2.shape[-1]
        if K2 != K2b:
            raise ValueError(f"second product: inner dimensions differ: {K2} vs {K2b}")
        la2, sa2, _ = _ld_stride(A2)
        lb2, sb2, _ = _ld_stride(B2)
        d.K2 = K2
        d.A2, d.lda2, d.stride_a2, d.a2_mn_major = A2.data_ptr(), la2, sa2, int(a2_mn)
        d.B2, d.ldb2, d.stride_b2, d.b2_mn_major = B2.data_ptr(), lb2, sb2, int(b2_mn)
    st = None if status is None else status.data_ptr()
    _lib.call("fdtd_gemm_bf16", C.byref(d), st, _lib.stream_ptr())
    return out
