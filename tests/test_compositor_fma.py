"""RTX_OPT_COMPOSITOR_FMA: the register-blocked filters with each tap's
multiply and add fused, against the oracle (RenderToy's rounding).

A fused tap rounds once where the reference rounds twice, so each output can
move by a few ulps of the running sum; a sum of positive and negative taps
can cancel, so the bound is relative to the magnitude of what was summed:
|gpu - oracle| <= 1e-5 * S per pixel and channel, S = the same filter applied
to |image| with |kernel| (for the two-pass blur, S is the blur of |image|;
for bloom, |image| + that blur).  Non-finite pixels (the NaN and infinite
values renders can hold) must land where the oracle's do.  The shapes cross
the kernels' tiles as the bit-exact compositor tests do.  The default (option
off) stays bit-exact: tests/test_gpu_parity.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(gpu, orc, bound, what):
    fin = np.isfinite(orc)
    assert np.array_equal(np.isnan(gpu), np.isnan(orc)), what
    assert np.array_equal(gpu[~fin & ~np.isnan(orc)], orc[~fin & ~np.isnan(orc)]), what
    ok = np.isfinite(gpu) & fin & np.isfinite(bound)
    err = np.abs(gpu[ok].astype(np.float64) - orc[ok])
    tol = 1e-5 * bound[ok].astype(np.float64) + 1e-30
    worst = float((err / tol).max()) if err.size else 0.0
    print(f"{what}: max |err| / (1e-5 S) = {worst:.3f}, bit-equal {np.mean(gpu[ok] == orc[ok]) * 100:.1f} %")
    assert worst <= 1.0, what


@pytest.mark.parametrize("shape", [(131, 2061), (1, 1030), (70, 9), (200, 1024), (1024, 1024)])
def test_fused_filters_within_tolerance(ctx, oracle, shape):
    import rendertoy_gb300 as rt
    H, W = shape
    rng = np.random.RandomState(H * 31 + W)
    img = rng.exponential(0.7, (H, W, 3)).astype(np.float32)
    img[rng.uniform(size=(H, W)) < 0.3] *= -1.0  # signed pixels: taps that cancel
    flat = img.reshape(-1, 3)
    bad = rng.choice(H * W, size=max(1, H * W // 997), replace=False)
    flat[bad[::2], 0] = np.nan
    flat[bad[1::2], 2] = np.inf
    absimg = np.abs(img)
    k5 = rng.normal(0, 1, (5, 5)).astype(np.float32)
    k3 = rng.normal(0, 1, (3, 3)).astype(np.float32)
    ctx.set_option(rt.OPT_COMPOSITOR_FMA, 1)
    try:
        for name, fn, bound in (
                ("blur49", lambda c: c.gaussian_blur(img, 49, 8.0), oracle.gaussian_blur(absimg, 49, 8.0)),
                ("blur7", lambda c: c.gaussian_blur(img, 7, 1.5), oracle.gaussian_blur(absimg, 7, 1.5)),
                ("bloom17", lambda c: c.bloom(img, 17, 3.0, 1.0), absimg + oracle.gaussian_blur(absimg, 17, 3.0)),
                ("conv5", lambda c: c.convolve(img, k5), oracle.convolve(absimg, np.abs(k5))),
                ("conv5_abs", lambda c: c.convolve(img, k5, absval=True), oracle.convolve(absimg, np.abs(k5))),
                ("conv3", lambda c: c.convolve(img, k3), oracle.convolve(absimg, np.abs(k3)))):
            _check(fn(ctx), fn(oracle), bound, f"{shape} {name}")
    finally:
        ctx.set_option(rt.OPT_COMPOSITOR_FMA, 0)
    # with the option off the same call is bit-exact again
    a, b = ctx.gaussian_blur(img, 7, 1.5), oracle.gaussian_blur(img, 7, 1.5)
    nan = np.isnan(b)
    assert np.array_equal(np.isnan(a), nan)
    assert np.array_equal(a[~nan].view(np.uint32), b[~nan].view(np.uint32))
