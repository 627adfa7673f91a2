"""Split-BF16 tensor-core GEMM against an FP64 product.

Bounds per element, with S = |A| |B|^T:
  2 pieces: |C - A B^T| <= 6e-5 S + 1e-6 |A B^T|  (~16 bits kept per operand,
            dropped p1q1 term: ~2^-16 relative per product)
  3 pieces: |C - A B^T| <= 2e-6 S + 1e-6 |A B^T|  (~24 bits per operand; the
            FP32 accumulator, ~K 2^-24 at worst, dominates)
  precise:  |C - A B^T| <= 1e-7 S + 1e-7 |A B^T|  (eight products, FP64 sums of
            once-rounded slab products; the FP32 output rounding is 6e-8)
"""
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(128, 128, 64), (200, 300, 100), (64, 1000, 640), (1000, 560, 640), (7, 5, 3), (333, 129, 1216)]


@pytest.fixture(scope="module")
def L():
    from openlowdin_gb300 import build, lint
    build.build()
    return lint


@pytest.mark.parametrize("pieces,rel", [(2, 6e-5), (3, 2e-6)])
@pytest.mark.parametrize("M,N,K", SHAPES)
def test_gemm_split_matches_fp64(L, M, N, K, pieces, rel):
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(M * 7919 + N * 31 + K)
    A = torch.randn(M, K, device="cuda", generator=g, dtype=torch.float32)
    B = torch.randn(N, K, device="cuda", generator=g, dtype=torch.float32) * 1e-3
    C = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    L.gemm_bf16_split(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K, pieces,
                      stream=torch.cuda.current_stream().cuda_stream)
    ref = A.double() @ B.double().T
    bound = rel * (A.double().abs() @ B.double().abs().T) + 1e-6 * ref.abs()
    err = (C.double() - ref).abs()
    assert torch.isfinite(C).all()
    assert bool((err <= bound).all()), float((err / bound).max())


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_gemm_precise_matches_fp64(L, M, N, K):
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(M * 13 + N * 7 + K)
    A = torch.randn(M, K, device="cuda", generator=g, dtype=torch.float32)
    B = torch.randn(N, K, device="cuda", generator=g, dtype=torch.float32) * 1e3
    C = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    L.gemm_bf16_precise(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K,
                        stream=torch.cuda.current_stream().cuda_stream)
    ref = A.double() @ B.double().T
    bound = 1e-7 * (A.double().abs() @ B.double().abs().T) + 1e-7 * ref.abs()
    err = (C.double() - ref).abs()
    assert torch.isfinite(C).all()
    assert bool((err <= bound).all()), float((err / bound).max())


def test_gemm_precise_is_unbiased(L):
    """Positive operands: every partial sum has one sign, so a systematic
    rounding direction shows as a mean relative error of the order of the
    FP32 unit (-3.3e-8 with 32-wide slabs, -1.3e-8 with 16-wide slabs and no
    compensation of the tensor cores' rounding losses); the mean must stay well
    below the output rounding's spread (3e-8)."""
    torch = pytest.importorskip("torch")
    M, N, K = 128, 4096, 640
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.rand(M, K, device="cuda", generator=g, dtype=torch.float32)
    B = torch.rand(N, K, device="cuda", generator=g, dtype=torch.float32)
    C = torch.empty((M, N), device="cuda", dtype=torch.float32)
    L.gemm_bf16_precise(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K,
                        stream=torch.cuda.current_stream().cuda_stream)
    ref = A.double() @ B.double().T
    rel = (C.double() - ref) / ref
    assert abs(float(rel.mean())) < 5e-9, float(rel.mean())
