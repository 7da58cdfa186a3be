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


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (200, 144, 96), (40, 16, 8), (256, 304, 200)])
@pytest.mark.parametrize("a_mn,b_mn", [(False, False), (True, False), (False, True), (True, True)])
def test_gemm_bf16(ctx, M, N, K, a_mn, b_mn):
    rng = np.random.RandomState(M + N + K)
    A = to_bf16(rng.normal(size=(M, K)))
    B = to_bf16(rng.normal(size=(N, K)))
    Aa = np.ascontiguousarray(A.T) if a_mn else A
    Bb = np.ascontiguousarray(B.T) if b_mn else B
    C = ctx.gemm_bf16(Aa, Bb, a_mn=a_mn, b_mn=b_mn)
    ref = from_bf16(A).astype(np.float64) @ from_bf16(B).astype(np.float64).T
    err = np.abs(C - ref).max() / max(np.abs(ref).max(), 1e-6)
    assert err < 1e-5, err
