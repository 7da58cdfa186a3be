"""Procedural textures (RenderToy src/procedural.cpp:8-46) bound to materials.

CPU: the oracle's samplers against RenderToy's own CheckerBoard / Wave /
PerlinNoise::Sample outputs (tests/golden/textures.npz, with the permutation
a default-constructed PerlinNoise uses), bit for bit; the scene generator.
GPU: the device samplers against the same vectors (bit for bit; Wave within
1e-6 for the sine); a textured procedural scene per path (1e-4 relative) and
in the albedo pass against the oracle.
"""
import numpy as np
import pytest

from helpers import rel_close
from rendertoy_gb300 import scenes


def _cases(golden):
    g = golden("textures")
    for i, (k, p) in enumerate(zip(g["kinds"], g["params"])):
        yield int(k), float(p), g[f"out{i}"], g


def test_oracle_samplers_match_reference(oracle, golden):
    for k, p, want, g in _cases(golden):
        got = oracle.texture_sample(k, p, g["uv"], perm=g["perm"])
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (k, p)


def test_procedural_scene_generator():
    sc, job = scenes.procedural_scene(3)
    assert sc.n_tris > 1000 and 1 <= job["n_lights"] <= 4
    assert 1 <= job["spp"] <= 64 and (job["W"], job["H"]) in [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    assert len(sc.emitters()) == 2 * job["n_lights"]
    kinds = sc.mats[:, 21]
    assert set(np.unique(kinds)).issubset({0.0, 1.0, 2.0, 3.0})
    sc2, job2 = scenes.procedural_scene(3)
    assert np.array_equal(sc.verts, sc2.verts) and job == job2
    # blackbody colours are normalised to a maximum of 1, reddish when cool
    c = scenes.blackbody_rgb(2500.0)
    assert abs(c.max() - 1.0) < 1e-12 and c[0] > c[1] > c[2]


@pytest.mark.gpu
def test_device_samplers_match_reference(ctx, golden):
    g = golden("textures")
    ctx.set_texture_table(g["perm"])
    try:
        for k, p, want, _ in _cases(golden):
            got = ctx.texture_sample(k, p, g["uv"])
            if k == 2:
                assert np.abs(got - want).max() <= 1e-6, (k, p)
            else:
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (k, p)
    finally:
        ctx.set_texture_table(_default_table(ctx))


def _default_table(ctx):
    """include/rtx.h's default table: Fisher-Yates driven by splitmix64."""
    p = np.arange(256, dtype=np.uint8)
    x = 0
    m = (1 << 64) - 1
    for i in range(255, 0, -1):
        x = (x + 0x9E3779B97F4A7C15) & m
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        z ^= z >> 31
        j = z % (i + 1)
        p[i], p[j] = p[j], p[i]
    return p


@pytest.mark.gpu
def test_textured_scene_matches_oracle(ctx, oracle, golden):
    sc, _ = scenes.procedural_scene(11, n_tris=3000)
    assert (sc.mats[:, 21] != 0).sum() >= 2
    perm = golden("textures")["perm"]
    ctx.upload(sc)
    ctx.set_texture_table(perm)
    osc = oracle.scene(sc)
    osc.set_texture_table(perm)
    try:
        W, H = 40, 32
        near, far = float(sc.camera[19]), float(sc.camera[20])
        _, a, _ = ctx.aov(W, H, near, far)
        _, ra, _ = osc.aov(W, H, near, far)
        assert rel_close(a, ra.reshape(a.shape), 1e-6, 1e-7).all()
        got = ctx.trace_paths(W, H, 0, 2, 6, seed=3)
        ref = osc.trace_paths(W, H, 0, 2, 6, 3)
        ok = rel_close(got, ref, 1e-4, 1e-6).all(-1)
        assert ok.mean() >= 0.99, ok.mean()
    finally:
        ctx.set_texture_table(_default_table(ctx))
        osc.close()


@pytest.mark.gpu
def test_texture_table_must_be_a_permutation(ctx):
    import rendertoy_gb300 as rt
    with pytest.raises(rt.RtxError):
        ctx.set_texture_table(np.zeros(256, np.uint8))
    with pytest.raises(rt.RtxError):
        ctx.texture_sample(4, 1.0, np.zeros((4, 2), np.float32))
