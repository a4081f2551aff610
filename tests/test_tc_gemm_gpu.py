"""BF16 tensor-core GEMM (tcgen05 + TMA + TMEM) against a plain PyTorch FP32
matmul of the same BF16 operands: K-major and MN-major operands, batches,
batch-shared operands, ragged sizes and the fused epilogue."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float((a.float() - b).abs().max() / b.abs().max().clamp_min(1e-30))


@pytest.mark.parametrize("a_mn", [False, True])
@pytest.mark.parametrize("b_mn", [False, True])
@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (304, 200, 136), (512, 64, 2048), (136, 256, 72)])
def test_gemm_layouts(cuda_lib, a_mn, b_mn, M, N, K):
    from simulation_gb300 import tc
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).bfloat16()
    B = torch.randn(N, K, device="cuda", generator=g).bfloat16()
    Ain = A.T.contiguous() if a_mn else A
    Bin = B.T.contiguous() if b_mn else B
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    C = tc.gemm(Ain, Bin, a_mn=a_mn, b_mn=b_mn, status=st)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert _rel(C, A.float() @ B.float().T) <= 1e-5


def test_gemm_batched_shared_and_epilogue(cuda_lib):
    from simulation_gb300 import tc
    g = torch.Generator(device="cuda").manual_seed(7)
    nb, M, N, K = 5, 256, 128, 192
    A = torch.randn(nb, K, M, device="cuda", generator=g).bfloat16()      # MN-major per batch
    Bs = torch.randn(N, K, device="cuda", generator=g).bfloat16()        # shared K-major B
    bias = torch.randn(N, device="cuda", generator=g)
    res = torch.randn(nb, M, N, device="cuda", generator=g).bfloat16()
    pre = torch.empty(nb, M, N, device="cuda", dtype=torch.bfloat16)
    out = tc.gemm(A, Bs.unsqueeze(0).expand(nb, -1, -1), a_mn=True, out_dtype=torch.bfloat16, bias=bias,
                  residual=res, gelu=True, pre=pre, alpha=0.5)
    torch.cuda.synchronize()
    z = 0.5 * (A.float().transpose(1, 2) @ Bs.float().T) + bias + res.float()
    assert _rel(pre, z) <= 1e-2
    assert _rel(out, torch.nn.functional.gelu(z, approximate="tanh")) <= 1e-2
    acc = torch.randn(nb, M, N, device="cuda", generator=g)
    ref = acc + A.float().transpose(1, 2) @ Bs.float().T
    tc.gemm(A, Bs.unsqueeze(0).expand(nb, -1, -1), a_mn=True, out=acc, accumulate=True)
    torch.cuda.synchronize()
    assert _rel(acc, ref) <= 1e-5


def test_gemm_rejects_unaligned_leading_dimension(cuda_lib):
    """TMA needs 16-byte row strides: an MN-major A with M = 300 (600-byte rows)
    is refused on the host before any launch."""
    from simulation_gb300 import _lib, tc
    A = torch.zeros(64, 300, device="cuda", dtype=torch.bfloat16)
    B = torch.zeros(128, 64, device="cuda", dtype=torch.bfloat16)
    with pytest.raises(_lib.FdtdError) as e:
        tc.gemm(A, B, a_mn=True)
    assert e.value.code == -3


def test_gemm_second_product_shares_the_accumulator(cuda_lib):
    """acc = A.B^T + A2.B2' with a batched A, a shared B, a shared MN-major A2
    and a batched B2, then bias + GELU: the fused inverse-DFT + pointwise layer."""
    from simulation_gb300 import tc
    g = torch.Generator(device="cuda").manual_seed(11)
    nb, M, N, K, K2 = 3, 256, 128, 128, 64
    A = torch.randn(nb, M, K, device="cuda", generator=g).bfloat16()
    W = torch.randn(N, K, device="cuda", generator=g).bfloat16()
    A2t = torch.randn(K2, M, device="cuda", generator=g).bfloat16()     # stored transposed
    B2 = torch.randn(nb, N, K2, device="cuda", generator=g).bfloat16()
    bias = torch.randn(N, device="cuda", generator=g)
    out = tc.gemm(A, W, bias=bias, gelu=True, out_dtype=torch.bfloat16, second=(A2t, B2, True, False))
    torch.cuda.synchronize()
    z = A.float() @ W.float().T + A2t.float().T @ B2.float().transpose(1, 2) + bias
    assert _rel(out, torch.nn.functional.gelu(z, approximate="tanh")) <= 1e-2
