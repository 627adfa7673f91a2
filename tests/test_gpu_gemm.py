"""3-term split-BF16 tensor-core GEMM against an FP64 product.

Bound per element: |C - A B^T| <= 6e-5 (|A| |B|^T) + 1e-6 |A B^T|: the
two-term BF16 representation keeps about 16 bits of each operand (the dropped
lo*lo term and the rounding of hi and lo give ~2^-16 relative per product) and
the FP32 accumulator adds ~K 2^-24.
"""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from openlowdin_gb300 import build, lint
    build.build()
    return lint


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (200, 300, 100), (64, 1000, 640), (1000, 560, 640),
                                   (7, 5, 3), (333, 129, 1216)])
def test_gemm_bf16x3_matches_fp64(L, M, N, K):
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(M * 7919 + N * 31 + K)
    A = torch.randn(M, K, device="cuda", generator=g, dtype=torch.float32)
    B = torch.randn(N, K, device="cuda", generator=g, dtype=torch.float32) * 1e-3
    C = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    L.gemm_bf16x3(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K,
                  stream=torch.cuda.current_stream().cuda_stream)
    ref = A.double() @ B.double().T
    bound = 6e-5 * (A.double().abs() @ B.double().abs().T) + 1e-6 * ref.abs()
    err = (C.double() - ref).abs()
    assert torch.isfinite(C).all()
    assert bool((err <= bound).all()), float((err / bound).max())
