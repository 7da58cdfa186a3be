"""Display resolve (Image::Tonemap, Image::GammaCorrection) and the BMP / PPM
exporters (RenderToy include/RenderToy/compositor.h:220-226,
src/compositor.cpp:94-100, src/exporter.cpp:8-95).

CPU: the oracle against RenderToy's own outputs (tests/golden/resolve.npz),
bit / byte exact.  GPU: the device resolve against the same vectors (tonemap
bit-exact; gamma through powf within 2 ulp), the encoders byte-exact, and the
resolve fused into the path tracer's last accumulation equal to resolving its
output afterwards.
"""
import numpy as np
import pytest

from helpers import rel_close
from rendertoy_gb300 import scenes


def test_oracle_matches_reference(oracle, golden):
    g = golden("resolve")
    for tag, limit, gamma in (("tm", 1.5, 0.0), ("gm", 0.0, 2.2), ("tmgm", 1.5, 2.2), ("tmgm2", 4.0, 1.8)):
        got = oracle.tonemap_gamma(g["img"], limit, gamma)
        assert np.array_equal(np.nan_to_num(got, nan=-1).view(np.uint32),
                              np.nan_to_num(g[tag], nan=-1).view(np.uint32)), tag
    assert oracle.encode(g["enc_in"], True) == g["bmp"].tobytes()
    assert oracle.encode(g["enc_in"], False) == g["ppm"].tobytes()


def test_oracle_bmp_padding():
    """Rows of a width that is not a multiple of 4 are zero-padded and the
    header's size counts the padding (the reference writes the padding from a
    null pointer)."""
    from oracle import bind
    o = bind.load("oracle")
    img = np.full((2, 5, 3), 0.5, np.float32)
    b = o.encode(img, True)
    row = (5 * 3 + 3) & ~3
    assert len(b) == 54 + 2 * row and int.from_bytes(b[2:6], "little") == len(b)
    assert b[54 + 15:54 + row] == b"\x00" * (row - 15)


@pytest.mark.gpu
def test_device_resolve_matches_reference(ctx, golden):
    g = golden("resolve")
    img = g["img"]
    tm = ctx.tonemap(img, 1.5)
    assert np.array_equal(np.nan_to_num(tm, nan=-1).view(np.uint32), np.nan_to_num(g["tm"], nan=-1).view(np.uint32))
    for tag, limit, gamma in (("gm", 0.0, 2.2), ("tmgm", 1.5, 2.2), ("tmgm2", 4.0, 1.8)):
        disp, _ = ctx.resolve(img, limit, gamma, want_bytes=False)
        assert rel_close(disp, g[tag], 2.5e-7).all(), tag
    assert ctx.encode_bmp(g["enc_in"]) == g["bmp"].tobytes()
    assert ctx.encode_ppm(g["enc_in"]) == g["ppm"].tobytes()


@pytest.mark.gpu
def test_bytes_formats_and_nan(ctx):
    img = np.array([[[np.nan, 0.5, 2.0], [-1.0, 0.0, 1.0], [0.25, 0.75, 0.999]]], np.float32)
    _, rgb = ctx.resolve(img, 0.0, 0.0, fmt=1, want_display=False)
    q = lambda x: int(255.99 * min(max(x, 0.0), 1.0))  # noqa: E731
    assert list(rgb) == [0, q(0.5), 255, 0, 0, 255, q(0.25), q(0.75), q(0.999)]
    _, bgr = ctx.resolve(img, 0.0, 0.0, fmt=0, want_display=False)
    assert len(bgr) == 12 and list(bgr[:9]) == [255, q(0.5), 0, 255, 0, 0, q(0.999), q(0.75), q(0.25)]
    assert list(bgr[9:]) == [0, 0, 0]


@pytest.mark.gpu
def test_resolve_fused_into_render(ctx):
    ctx.upload(scenes.cornell_box())
    W, H = 50, 30  # a BMP row of 150 bytes + 2 padding
    plain = ctx.render_pt(W, H, 4, 6, seed=2)
    rad, disp, byt = ctx.render_pt_resolved(W, H, 4, 6, seed=2, limit=1.5, gamma=2.2, fmt=0)
    assert np.array_equal(rad.view(np.uint32), plain.view(np.uint32))
    d2, b2 = ctx.resolve(plain, 1.5, 2.2, fmt=0)
    assert np.array_equal(np.nan_to_num(disp, nan=-1), np.nan_to_num(d2, nan=-1))
    assert np.array_equal(byt, b2)
    rows = byt.reshape(H, -1)
    assert rows.shape[1] == 152 and not rows[:, 150:].any()
