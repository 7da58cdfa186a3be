"""The denoiser's tcgen05 GEMM engine (BF16 in, FP32 accumulation in TMEM)
against a float64 product of the same BF16 values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16(x):
    """float32 -> BF16 bits, round to nearest even."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def from_bf16(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (200, 144, 96), (37, 16, 8), (256, 300, 200)])
def test_gemm_bf16(ctx, M, N, K):
    rng = np.random.RandomState(M + N + K)
    A = to_bf16(rng.normal(size=(M, K)))
    B = to_bf16(rng.normal(size=(N, K)))
    C = ctx.gemm_bf16(A, B)
    ref = from_bf16(A).astype(np.float64) @ from_bf16(B).astype(np.float64).T
    err = np.abs(C - ref).max() / max(np.abs(ref).max(), 1e-6)
    assert err < 1e-5, err
