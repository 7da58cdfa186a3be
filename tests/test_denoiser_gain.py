"""What the trained denoiser gains over the method without it.

The network is trained briefly on pairs the renderer generates from
procedural scenes (4-spp radiance + albedo / normal / depth passes + spp ->
256-spp radiance), then run on held-out scenes: its output must be closer to
a 1024-spp render than the 4-spp input it was given (relMSE, eps 1e-2) by at
least 2x, and training must lower the loss.
"""
import numpy as np
import pytest

from rendertoy_gb300 import denoise as D
from rendertoy_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_trained_network_beats_its_input(ctx):
    ctx.dn_init(5)
    X, Y = D.make_pairs(ctx, range(16), W=128, H=128, in_spp=4, target_spp=256, max_depth=6,
                        tri_range=(1e3, 2e4), log=None)
    losses, _ = D.train(ctx, X, Y, 300, batch=8, crop=128, lr=1e-3, log=None)
    assert losses[-50:].mean() < 0.8 * losses[:50].mean()
    gains = []
    for s in (1000, 1001):
        sc, _ = scenes.procedural_scene(s, tri_range=(1e3, 2e4))
        ctx.upload(sc)
        rad = ctx.render_pt(128, 128, 4, 6, seed=7)
        a, n, d = D.frame_passes(ctx, sc, 128, 128)
        den = ctx.denoise(rad, a, n, d, 4)
        ref = ctx.render_pt(128, 128, 1024, 6, seed=8)
        e_in, _ = D.relmse(rad, ref)
        # the renders may hold RenderToy's NaN paths (relmse masks them); the
        # network's output may not
        assert np.isfinite(den).all()
        e_dn, _ = D.relmse(den, ref)
        gains.append(e_in / e_dn)
    print("relMSE gain of the denoised 4-spp frame over its input:", gains)
    assert min(gains) >= 2.0, gains
