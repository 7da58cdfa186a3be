"""Multi-scene batches: several scenes merged into one set of device arrays,
frames of uneven size and spp over them traced through one wavefront
(rtx_batch_upload / rtx_render_batch).

Each frame's random stream is the one a single render of its scene, camera
and seed uses, so every frame of a batch must equal that render bit for bit;
CUDA-graph replay (RTX_OPT_GRAPH) must equal direct launches for new seeds
and cameras.
"""
import numpy as np
import pytest

import rendertoy_gb300 as rt
from rendertoy_gb300 import scenes

pytestmark = pytest.mark.gpu


def _scenes():
    out = [scenes.cornell_box(), scenes.cornell_mixed()]
    for s in (5, 6):
        sc, _ = scenes.procedural_scene(s, tri_range=(2e3, 3e4))
        out.append(sc)
    return out


JOBS = [dict(scene=0, W=48, H=40, spp=3, seed=1), dict(scene=2, W=64, H=32, spp=2, seed=2),
        dict(scene=1, W=33, H=17, spp=5, seed=3), dict(scene=3, W=40, H=40, spp=1, seed=4),
        dict(scene=2, W=16, H=24, spp=4, seed=5)]


def _alone(ctx, sc, j, depth, camera=None):
    ctx.upload(sc)
    return ctx.render_pt(j["W"], j["H"], j["spp"], depth, seed=j["seed"], camera=camera)


def test_batch_frames_equal_single_renders(ctx):
    sc = _scenes()
    ctx.batch_upload(sc)
    imgs = ctx.render_batch(JOBS, 6)
    for j, img in zip(JOBS, imgs):
        ref = _alone(ctx, sc[j["scene"]], j, 6)
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), j


def test_batch_binary_and_wide_trees(ctx):
    """Frames equal single renders with the binary (0) and 4-wide (2) trees."""
    sc = _scenes()
    for trav in (0, 2):
        ctx.set_option(rt.OPT_TRAVERSAL, trav)
        try:
            ctx.batch_upload(sc)
            imgs = ctx.render_batch(JOBS[:3], 5)
            for j, img in zip(JOBS[:3], imgs):
                ref = _alone(ctx, sc[j["scene"]], j, 5)
                assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), (trav, j)
        finally:
            ctx.set_option(rt.OPT_TRAVERSAL, 2)


def test_batch_with_small_waves(ctx):
    """Waves that split frames and samples (64k paths) give the same images."""
    sc = _scenes()
    ctx.batch_upload(sc)
    a = ctx.render_batch(JOBS, 5)
    ctx.set_option(rt.OPT_WAVE_PATHS, 1 << 16)
    try:
        b = ctx.render_batch(JOBS, 5)
    finally:
        ctx.set_option(rt.OPT_WAVE_PATHS, 0)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_graph_replay(ctx):
    sc = _scenes()
    ctx.batch_upload(sc)
    ctx.set_option(rt.OPT_GRAPH, 1)
    try:
        ctx.render_batch(JOBS, 6)  # renders and captures
        jobs2 = [dict(j, seed=j["seed"] + 100) for j in JOBS]
        cam = sc[0].camera.copy()
        cam[3] += 10.0  # move frame 0's camera
        jobs2[0]["camera"] = cam
        got = ctx.render_batch(jobs2, 6)  # replays the graph with the new job table
        assert ctx.stats()["kernel_launches"] == 0
    finally:
        ctx.set_option(rt.OPT_GRAPH, 0)
    for j, img in zip(jobs2, got):
        ref = _alone(ctx, sc[j["scene"]], j, 6, camera=j.get("camera"))
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), j


def test_batch_errors(ctx):
    sc = _scenes()
    ctx.batch_upload(sc[:2])
    with pytest.raises(rt.RtxError):
        ctx.render_batch([dict(scene=2, W=8, H=8, spp=1)], 4)
    with pytest.raises(rt.RtxError):
        ctx.render_batch([dict(scene=0, W=8, H=8, spp=0)], 4)
    with rt.Context(0) as fresh:
        with pytest.raises(rt.RtxError):
            fresh.render_batch([dict(scene=0, W=8, H=8, spp=1, camera=sc[0].camera)], 4)


def test_material_sort_keeps_images(ctx):
    """RTX_OPT_SORT_MATERIAL reorders only which paths share a warp: single
    renders and batches are bit-identical with and without it."""
    sc = _scenes()
    ctx.upload(sc[1])
    a = ctx.render_pt(48, 40, 4, 6, seed=9)
    ctx.batch_upload(sc)
    ba = ctx.render_batch(JOBS, 6)
    ctx.set_option(rt.OPT_SORT_MATERIAL, 1)
    try:
        ctx.upload(sc[1])
        b = ctx.render_pt(48, 40, 4, 6, seed=9)
        ctx.batch_upload(sc)
        bb = ctx.render_batch(JOBS, 6)
    finally:
        ctx.set_option(rt.OPT_SORT_MATERIAL, 0)
        ctx.set_option(rt.OPT_TRAVERSAL, 2)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    for x, y in zip(ba, bb):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_autotune(ctx):
    sc = _scenes()
    ctx.batch_upload(sc)
    jobs = [dict(j, spp=j["spp"] * 4) for j in JOBS]
    try:
        res = ctx.batch_autotune(jobs, 6, scene_list=sc)
        assert res["trials"] >= 10 and res["ms"] <= res["ms_default"]
        assert ctx.get_option(rt.OPT_SORT_MATERIAL) == res["sort_material"]
        assert ctx.get_option(rt.OPT_SORT_RAYS) == res["sort_rays"]
        assert ctx.get_option(rt.OPT_OVERLAP) == res["overlap"]
        assert ctx.get_option(rt.OPT_TRAVERSAL) == res["traversal"] and res["traversal"] in (0, 2)
        assert res["leaf_size"] in (2, 4, 8) and res["block"] in (64, 128)
        assert ctx.get_option(rt.OPT_BLOCK) == res["block"]
        assert ctx.get_option(rt.OPT_LEAF_SIZE) == res["leaf_size"]
        # the tuned batch still renders the same images as single renders
        img = ctx.render_batch(jobs[:1], 6)[0]
        ref = _alone(ctx, sc[jobs[0]["scene"]], jobs[0], 6)
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    finally:
        ctx.set_option(rt.OPT_BLOCK, 128)
        ctx.set_option(rt.OPT_WAVE_PATHS, 0)
        ctx.set_option(rt.OPT_LEAF_SIZE, 4)
        ctx.set_option(rt.OPT_OVERLAP, 1)
        ctx.set_option(rt.OPT_SORT_MATERIAL, 0)
        ctx.set_option(rt.OPT_SORT_RAYS, 1)
        ctx.set_option(rt.OPT_TRAVERSAL, 2)


def test_overlap_does_not_change_results(ctx):
    """RTX_OPT_OVERLAP (each vertex's occlusion launch on a second stream
    beside the next vertex's closest-hit launch) changes only when kernels
    run: single renders, per-path traces, several waves per render and batch
    frames replayed from a CUDA graph are bit-identical with it on and off."""
    from helpers import same_bits
    sc = scenes.displaced_icosphere(subdiv=3)
    out = {}
    for ov in (0, 1):
        ctx.set_option(rt.OPT_OVERLAP, ov)
        try:
            ctx.upload(sc)
            a = ctx.trace_paths(40, 30, 0, 3, 12, seed=5)
            b = ctx.render_pt(64, 48, 6, 12, seed=5)
            ctx.set_option(rt.OPT_WAVE_PATHS, 1000)
            c = ctx.render_pt(64, 48, 3, 12, seed=6)
            ctx.set_option(rt.OPT_WAVE_PATHS, 0)
            ctx.batch_upload(_scenes())
            ctx.set_option(rt.OPT_GRAPH, 1)
            first = ctx.render_batch(JOBS, 6)
            replay = ctx.render_batch([dict(j, seed=j["seed"] + 10) for j in JOBS], 6)
            out[ov] = (a, b, c, first, replay)
        finally:
            ctx.set_option(rt.OPT_GRAPH, 0)
            ctx.set_option(rt.OPT_WAVE_PATHS, 0)
            ctx.set_option(rt.OPT_OVERLAP, 1)
    for x, y in zip(out[0][:3], out[1][:3]):
        assert same_bits(x, y)
    for frames_a, frames_b in zip(out[0][3:], out[1][3:]):
        for fa, fb in zip(frames_a, frames_b):
            assert same_bits(fa, fb)
