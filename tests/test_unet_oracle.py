"""The U-Net oracle's gradients against finite differences (FP64)."""
import numpy as np

from oracle import unet_oracle as U


def _fd(f, x, eps=1e-6):
    g = np.zeros_like(x)
    it = np.nditer(x, flags=["multi_index"])
    for _ in it:
        i = it.multi_index
        old = x[i]
        x[i] = old + eps
        a = f()
        x[i] = old - eps
        b = f()
        x[i] = old
        g[i] = (a - b) / (2 * eps)
    return g


def test_conv_gradients_match_finite_differences():
    rng = np.random.RandomState(0)
    x = rng.normal(size=(2, 5, 4, 3))
    w = rng.normal(size=(4, 3, 3, 3))
    b = rng.normal(size=4)
    r = rng.normal(size=(2, 5, 4, 4))
    loss = lambda: float((U.conv3x3(x, w, b) * r).sum())  # noqa: E731
    dx = U.conv3x3_dgrad(r, w)
    dw, db = U.conv3x3_wgrad(x, r)
    assert np.allclose(dx, _fd(loss, x), atol=1e-6)
    assert np.allclose(dw, _fd(loss, w), atol=1e-6)
    assert np.allclose(db, _fd(loss, b), atol=1e-6)


def test_pool_upsample_loss_adam():
    rng = np.random.RandomState(1)
    x = rng.normal(size=(1, 4, 6, 2))
    r = rng.normal(size=(1, 2, 3, 2))
    assert np.allclose(U.avgpool2_grad(r), _fd(lambda: float((U.avgpool2(x) * r).sum()), x))
    r2 = rng.normal(size=(1, 8, 12, 2))
    assert np.allclose(U.upsample2_grad(r2), _fd(lambda: float((U.upsample2(x) * r2).sum()), x))
    t = np.abs(rng.normal(size=x.shape))
    val, g = U.l1_log_loss(x, t)
    assert np.isclose(val, np.abs(x - np.log1p(t)).mean())
    assert np.allclose(g, _fd(lambda: U.l1_log_loss(x, t)[0], x), atol=1e-6)
    p, m, v = U.adam(np.ones(3), np.array([1.0, -2.0, 0.0]), np.zeros(3), np.zeros(3), 1)
    assert np.allclose(p, [1 - 3e-4, 1 + 3e-4, 1.0])
