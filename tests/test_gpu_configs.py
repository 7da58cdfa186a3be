"""The CUDA path at the two single-scene workloads' own sizes, against the
oracle (RenderToy's renderer restated, pinned to the reference's outputs).

* Cornell box: 256 x 256, 16 spp, max depth 8 -- every primary hit, every AOV
  pixel and every one of the 1,048,576 paths, plus the 1024-spp mean image of
  a 64 x 64 film.
* Displaced icosphere (1,310,720 + 12 triangles): 1024 x 1024, 64 spp, max
  depth 12 -- every primary hit and AOV pixel of the full film, 4,096 paths
  drawn across all 64 sample indices, and (a size-independent property of the
  whole benched frame) the 64-spp image equal, bit for bit, to the sample-order
  mean of its 64 per-path images.

Bars: primary-hit ids equal on >= 99.99 % of pixels with t within 1e-5
relative; AOVs within 1e-5; per-path radiance within 1e-4 relative on
>= 99.9 % of paths; mean image relMSE <= 1e-3 (eps 1e-2).
"""
import numpy as np
import pytest

from helpers import rel_close, relmse, same_bits
from rendertoy_gb300 import scenes

pytestmark = pytest.mark.gpu

CORNELL = dict(W=256, H=256, spp=16, depth=8)
ICO = dict(W=1024, H=1024, spp=64, depth=12)


def _check_primary_and_aov(ctx, osc, W, H, near, far, tag):
    tri, tuv = ctx.primary(W, H)
    rtri, rtuv = osc.primary(W, H)
    same = tri == rtri
    print(f"{tag}: primary ids equal on {same.mean() * 100:.4f} % of {same.size} pixels")
    assert same.mean() >= 0.9999, same.mean()
    assert rel_close(tuv[..., 0][same], rtuv[..., 0][same], 1e-5).all()
    n, a, d = ctx.aov(W, H, near, far)
    rn, ra, rd = osc.aov(W, H, near, far)
    for got, ref, key in ((n, rn, "normal"), (a, ra, "albedo"), (d, rd, "depth")):
        diff = np.abs(got - ref).max(-1)
        print(f"{tag}: {key} max |diff| {diff[same].max():.3g}")
        assert (diff[same] <= 1e-5).all(), (key, diff[same].max())


def test_cornell_config_size(ctx, oracle):
    sc = scenes.cornell_box()
    assert sc.n_tris == 36
    ctx.upload(sc)
    osc = oracle.scene(sc)
    W, H, spp, depth = CORNELL["W"], CORNELL["H"], CORNELL["spp"], CORNELL["depth"]
    _check_primary_and_aov(ctx, osc, W, H, float(sc.camera[19]), float(sc.camera[20]), "cornell")
    got = ctx.trace_paths(W, H, 0, spp, depth, seed=11)
    ref = osc.trace_paths(W, H, 0, spp, depth, 11)
    ok = rel_close(got, ref, 1e-4, atol=1e-6).all(-1)
    print(f"cornell depth {depth}: {ok.mean() * 100:.4f} % of {ok.size} paths within 1e-4")
    assert ok.mean() >= 0.999, ok.mean()
    # the rendered frame is the sample-order mean of exactly these paths
    img = ctx.render_pt(W, H, spp, depth, seed=11)
    acc = np.zeros((H * W, 3), np.float32)
    for s in range(spp):
        acc = acc + got[s] / np.float32(spp)
    assert same_bits(img.reshape(-1, 3), acc)


def test_cornell_mean_image_1024spp(ctx, oracle):
    sc = scenes.cornell_box()
    ctx.upload(sc)
    W = H = 64
    gpu = ctx.render_pt(W, H, 1024, CORNELL["depth"], seed=3)
    ref = oracle.scene(sc).render_pt(W, H, 1024, CORNELL["depth"], 3)
    e = relmse(gpu, ref)
    print(f"cornell 64x64 at 1024 spp: relMSE(gpu, oracle) = {e:.3g}")
    assert e <= 1e-3
    assert np.isfinite(gpu).mean() > 0.99


@pytest.fixture(scope="module")
def ico(ctx, oracle):
    sc = scenes.displaced_icosphere(subdiv=8)
    assert sc.n_tris == 20 * 4 ** 8 + 12
    return sc, oracle.scene(sc)


def test_icosphere_primary_and_aov_full_film(ctx, ico):
    sc, osc = ico
    ctx.upload(sc)
    _check_primary_and_aov(ctx, osc, ICO["W"], ICO["H"], float(sc.camera[19]), float(sc.camera[20]),
                           "icosphere")


def test_icosphere_paths_across_samples(ctx, ico):
    """4,096 paths of the benched frame: 16 sample indices spread over 0..63,
    256 random pixels each, at max depth 12."""
    sc, osc = ico
    ctx.upload(sc)
    W, H, depth, seed = ICO["W"], ICO["H"], ICO["depth"], 5
    rng = np.random.RandomState(7)
    samples = np.sort(rng.choice(ICO["spp"], 16, replace=False))
    oks = []
    for s in samples:
        pix = rng.choice(W * H, 256, replace=False).astype(np.int32)
        got = ctx.trace_paths(W, H, int(s), 1, depth, seed=seed).reshape(W * H, 3)[pix]
        ref = osc.trace_paths(W, H, int(s), 1, depth, seed, pixels=pix)[0]
        oks.append(rel_close(got, ref, 1e-4, 1e-6).all(-1))
    ok = np.concatenate(oks)
    print(f"icosphere depth {depth}: {ok.mean() * 100:.3f} % of {ok.size} paths within 1e-4 "
          f"(samples {samples.tolist()})")
    assert ok.mean() >= 0.999, ok.mean()


def test_icosphere_frame_is_mean_of_its_paths(ctx, ico):
    """The full benched frame (1024^2, 64 spp, depth 12) equals, bit for bit,
    the sample-order mean of its 64 per-path images: what the per-path checks
    establish for sampled paths holds for the accumulated frame."""
    import torch
    sc, _ = ico
    ctx.upload(sc)
    W, H, spp, depth, seed = ICO["W"], ICO["H"], ICO["spp"], ICO["depth"], 21
    img = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    ctx.render_pt(W, H, spp, depth, seed=seed, out=img)
    ctx.synchronize()
    paths = torch.empty((1, H * W, 3), dtype=torch.float32, device="cuda")
    acc = torch.zeros((H * W, 3), dtype=torch.float32, device="cuda")
    n = torch.tensor(float(spp), dtype=torch.float32, device="cuda")
    for s in range(spp):
        ctx.trace_paths(W, H, s, 1, depth, seed=seed, out=paths)
        ctx.synchronize()
        acc = acc + paths[0] / n
        torch.cuda.synchronize()  # before the next trace overwrites `paths`
    a = img.reshape(-1, 3).cpu().numpy()
    b = acc.cpu().numpy()
    assert same_bits(a, b)
    assert np.isfinite(a).mean() > 0.999
