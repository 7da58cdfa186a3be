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
    p, m, v = U.adam(np.ones(3), np.array([1.0, -2.0, 0.0]), np.zeros(3), np.zeros(3), 1)
    assert np.allclose(p, [1 - 3e-4, 1 + 3e-4, 1.0])


def test_kernel_predicting_loss():
    """The filtered radiance is a convex combination of the 5 x 5 taps
    (clamped at the frame's edge); the loss gradient with respect to the
    logits matches central differences of the loss with its denominator held
    at the base point's output; NaN / infinite radiance is made safe."""
    rng = np.random.RandomState(2)
    logits = rng.normal(size=(2, 6, 5, 32))
    raw = rng.uniform(0, 2, (2, 6, 5, 11))
    raw[0, 0, 0, 0] = np.nan
    raw[1, 2, 3, 1] = np.inf
    t = rng.uniform(0, 2, (2, 6, 5, 3))
    o = U.kp_apply(logits, raw)
    assert np.isfinite(o).all()
    rad = U.sane(raw[..., :3])
    assert (o <= rad.max() + 1e-9).all() and (o >= 0).all()
    # a filter that puts all weight on the centre tap returns the input
    centre = np.full((2, 6, 5, 32), -60.0)
    centre[..., 12] = 60.0
    assert np.allclose(U.kp_apply(centre, raw), rad)
    # the corner pixel's up-left tap is clamped onto the corner itself
    corner = np.full((2, 6, 5, 32), -60.0)
    corner[..., 0] = 60.0
    assert np.allclose(U.kp_apply(corner, raw)[:, 0, 0], rad[:, 0, 0])
    loss, g = U.kp_loss(logits, raw, t)
    den = o * o + U.REL_EPS
    assert np.isclose(loss, ((o - t) ** 2 / den).mean())
    assert (g[..., 25:] == 0).all()
    fd = _fd(lambda: float(((U.kp_apply(logits, raw) - t) ** 2 / den).mean()), logits)
    assert np.allclose(g, fd, atol=1e-9)


def test_bf16_rounding_is_nearest_even():
    e = 2.0 ** -7  # BF16 spacing at 1.0 (7 stored mantissa bits)
    vals = np.array([1.0, 1 + e / 2, 1 + 3 * e / 2, 1 + e / 2 + 1e-6, -2.5, 0.0, 3.0e38])
    got = U.to_bf16(vals)
    assert got[0] == 1.0 and got[1] == 1.0  # tie -> even
    assert got[2] == 1 + 2 * e               # tie -> even (upwards)
    assert got[3] == 1 + e                   # above the tie
    assert got[4] == -2.5 and got[5] == 0.0
    assert np.isfinite(got[6])


def test_layer_table_layout():
    rows, n = U.layer_table()
    assert len(rows) == 14
    end = 0
    for r in rows:
        assert r["w_off"] % 4 == 0 and r["b_off"] % 4 == 0 and r["w_off"] >= end
        assert r["cin_pad"] % 16 == 0 and r["cout_pad"] % 16 == 0
        end = r["b_off"] + r["cout_pad"]
    assert end <= n
    # 32 / 64 / 96 / 128 / 160 channels, about 1.3M parameters
    assert [r["cout"] for r in rows] == [32, 32, 64, 64, 96, 96, 128, 128, 160, 128, 96, 64, 32, 25]
    assert rows[0]["cin"] == 11 and rows[-1]["cout_pad"] == 32
    assert 1.2e6 < U.real_param_count() < 1.4e6


def test_network_gradients_match_finite_differences():
    """The whole U-Net (FP64, no rounding): the analytic gradient of the
    relative squared error of the filtered radiance (its denominator held at
    the base point's output) against central differences, for weights and
    biases of every layer."""
    rng = np.random.RandomState(3)
    p = U.init_params(5)
    rows, _ = U.layer_table()
    for r in rows:  # non-zero biases so that every bias gradient is exercised
        p[r["b_off"]:r["b_off"] + r["cout"]] = rng.normal(0, 0.05, r["cout"])
    raw = rng.uniform(0, 1, (1, 16, 16, 11))
    raw[..., :3] *= 4.0
    raw[..., 10] = 16.0
    target = rng.uniform(0, 3, (1, 16, 16, 3))
    net = U.UNet(p)
    loss, g = net.loss_and_grads(raw, target)
    assert np.isfinite(loss)
    o0 = U.UNet(p).denoise(raw)
    den = o0 * o0 + U.REL_EPS

    def f():
        return (((U.UNet(p).denoise(raw) - target) ** 2) / den).mean()

    picks = []
    for r in rows:
        w = r["w_off"]
        ci = r["cin"] if r["cin_pad"] == r["c1_pad"] else r["cin_pad"]
        for _ in range(2):
            o, t, c = rng.randint(r["cout"]), rng.randint(9), rng.randint(ci)
            picks.append(w + (o * 9 + t) * r["cin_pad"] + c)
        picks.append(r["b_off"] + rng.randint(r["cout"]))
    eps = 1e-6
    for k in picks:
        old = p[k]
        p[k] = old + eps
        a = f()
        p[k] = old - eps
        b = f()
        p[k] = old
        fd = (a - b) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(fd), (k, fd, g[k])
