"""CUDA path (librtx, through the C ABI) against the reference's golden vectors
and the oracle.

Bars (from the reference's own outputs, tests/golden):
  * primary-hit triangle ids equal on >= 99.99 % of pixels, hit t within 1e-5
    relative where they are equal;
  * normal / albedo / depth passes within 1e-5;
  * per-path radiance within 1e-4 relative on >= 99 % of paths (paths whose
    direction is decided by a transcendental rounded one ulp apart can take
    another branch; both renderers run the same Philox stream);
  * mean image at 1024 spp: relMSE against the oracle <= 1e-3;
  * compositor bit-exact (the sums run in the reference's order, unfused).
"""
import numpy as np
import pytest

from helpers import bits, rel_close, relmse, scene_from_fixture
from rendertoy_gb300 import scenes

pytestmark = pytest.mark.gpu

TAGS = ["cornell", "mixed"]


@pytest.fixture(scope="module")
def fixture_scene(ctx, golden):
    cache = {}

    def get(tag):
        g = golden(f"scene_{tag}")
        ctx.upload(scene_from_fixture(g))
        return g
    return get


@pytest.mark.parametrize("tag", TAGS)
def test_emitter_order(ctx, fixture_scene, tag):
    g = fixture_scene(tag)
    assert np.array_equal(ctx.emitters(), g["emitters"])


@pytest.mark.parametrize("tag", TAGS)
def test_primary_hits(ctx, fixture_scene, tag):
    g = fixture_scene(tag)
    W, H = int(g["W"]), int(g["H"])
    tri, tuv = ctx.primary(W, H)
    same = tri == g["primary_tri"]
    assert same.mean() >= 0.9999, same.mean()
    assert rel_close(tuv[..., 0][same], g["primary_tuv"][..., 0][same], 1e-5).all()
    # the exact Moller-Trumbore restatement reproduces t, u, v bit for bit
    assert (bits(tuv)[same] == bits(g["primary_tuv"])[same]).all(-1).mean() >= 0.9999


@pytest.mark.parametrize("tag", TAGS)
def test_aov(ctx, fixture_scene, tag):
    g = fixture_scene(tag)
    W, H = int(g["W"]), int(g["H"])
    near, far = float(g["camera"][19]), float(g["camera"][20])
    n, a, d = ctx.aov(W, H, near, far)
    same = ctx.primary(W, H)[0] == g["primary_tri"]
    for got, key in ((n, "aov_normal"), (a, "aov_albedo"), (d, "aov_depth")):
        diff = np.abs(got - g[key]).max(-1)
        assert (diff[same] <= 1e-5).all(), (key, diff.max())


@pytest.mark.parametrize("tag", TAGS)
@pytest.mark.parametrize("depth", [5, 8])
def test_per_path_radiance(ctx, fixture_scene, tag, depth):
    g = fixture_scene(tag)
    W, H = int(g["W"]), int(g["H"])
    ref = g[f"paths_d{depth}"]
    got = ctx.trace_paths(W, H, 0, ref.shape[0], depth, int(g["seed"]))
    ok = rel_close(got, ref, 1e-4, atol=1e-6).all(-1)
    print(f"{tag} depth {depth}: {ok.mean() * 100:.3f} % of {ok.size} paths within 1e-4")
    assert ok.mean() >= 0.99, ok.mean()


def test_intersect(ctx, golden):
    g = golden("intersect_mixed")
    ctx.upload(scenes.cornell_mixed())
    tri, tuv = ctx.intersect(g["rays"], g["exclude"])
    same = tri == g["tri"]
    assert same.mean() >= 0.9999, same.mean()
    assert (bits(tuv)[same] == bits(g["tuv"])[same]).all()


def test_compositor_bit_exact(ctx, golden, oracle):
    g = golden("compositor")
    for tag in ("a", "b"):
        img = g[f"img_{tag}"]
        k5 = g[f"k5_{tag}"]
        cases = {
            "blur7": (lambda c: c.gaussian_blur(img, 7, 1.5)),
            "blur49": (lambda c: c.gaussian_blur(img, 49, 8.0)),
            "edge": (lambda c: c.edge_detect(img)),
            "bloom": (lambda c: c.bloom(img, 9, 2.0, 0.8)),
        }
        for flags in ((0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0), (0, 1, 1)):
            cases["conv5_" + "".join(map(str, flags))] = (
                lambda c, f=flags: c.convolve(img, k5, normalize=f[0], length=f[1], absval=f[2]))
        for name, fn in cases.items():
            gpu, orc = fn(ctx), fn(oracle)
            assert np.array_equal(bits(gpu), bits(orc)), (tag, name)
            rows = g[f"rows_{name}_{tag}"]
            assert np.array_equal(bits(gpu[rows]), bits(g[f"{name}_{tag}"][rows])), (tag, name)


@pytest.mark.parametrize("shape", [(131, 2061), (1, 1030), (70, 9), (200, 1024)])
def test_compositor_tiles_nan_inf(ctx, oracle, shape):
    """Images that cross the kernels' tiles (rows of more than 1,024 pixels,
    columns of more than 64 rows, ragged edges, single rows) and carry the NaN
    and infinite pixels renders can hold: every filter still bit-exact, and a
    NaN spreads exactly as far as the reference's taps reach."""
    H, W = shape
    rng = np.random.RandomState(H * 7919 + W)
    img = rng.exponential(0.7, (H, W, 3)).astype(np.float32)
    flat = img.reshape(-1, 3)
    bad = rng.choice(H * W, size=max(1, H * W // 997), replace=False)
    flat[bad[::2], 0] = np.nan
    flat[bad[1::2], 2] = np.inf
    k5 = rng.normal(0, 1, (5, 5)).astype(np.float32)
    k3 = rng.normal(0, 1, (3, 3)).astype(np.float32)
    cases = {
        "blur49": lambda c: c.gaussian_blur(img, 49, 8.0),
        "blur7": lambda c: c.gaussian_blur(img, 7, 1.5),
        "blur2": lambda c: c.gaussian_blur(img, 2, 0.7),
        "bloom17": lambda c: c.bloom(img, 17, 3.0, 1.0),
        "conv5_abs": lambda c: c.convolve(img, k5, absval=True),
        "conv3_len": lambda c: c.convolve(img, k3, length=True),
        "conv3_norm": lambda c: c.convolve(img, k3, normalize=True),
    }
    for name, fn in cases.items():
        gpu, orc = fn(ctx), fn(oracle)
        # NaN payloads are not portable (the host propagates the input's, the
        # GPU writes its canonical NaN): NaN positions must agree, every other
        # value bit for bit
        nan = np.isnan(orc)
        assert np.array_equal(np.isnan(gpu), nan), (shape, name)
        assert np.array_equal(bits(gpu)[~nan], bits(orc)[~nan]), (shape, name)


def test_compositor_large_kernel(ctx, oracle):
    """Bloom(500, 50, 1) as RenderToy's Cornell demo applies it: a kernel wider
    than the image takes the direct path; still bit-exact."""
    rng = np.random.RandomState(0)
    img = rng.exponential(0.7, (40, 64, 3)).astype(np.float32)
    assert np.array_equal(bits(ctx.bloom(img, 101, 20.0, 1.0)), bits(oracle.bloom(img, 101, 20.0, 1.0)))
    assert np.array_equal(bits(ctx.gaussian_blur(img, 500, 50.0)),
                          bits(oracle.gaussian_blur(img, 500, 50.0)))


def test_mean_image_1024spp(ctx, oracle):
    sc = scenes.cornell_box()
    ctx.upload(sc)
    W = H = 24
    gpu = ctx.render_pt(W, H, 1024, 8, seed=3)
    ref = oracle.scene(sc).render_pt(W, H, 1024, 8, 3)
    e = relmse(gpu, ref)
    print("relMSE(gpu, oracle) at 1024 spp:", e)
    assert e <= 1e-3
    assert np.isfinite(gpu).mean() > 0.99


def test_accumulation_matches_paths(ctx):
    """render_pt == sum_s trace_paths(s) / spp, in sample order."""
    sc = scenes.cornell_box()
    ctx.upload(sc)
    W, H, spp = 16, 12, 5
    img = ctx.render_pt(W, H, spp, 6, seed=9)
    paths = ctx.trace_paths(W, H, 0, spp, 6, seed=9)
    acc = np.zeros((H * W, 3), np.float32)
    for s in range(spp):
        acc = acc + paths[s] / np.float32(spp)
    assert np.array_equal(bits(img.reshape(-1, 3)), bits(acc))


def test_waves_do_not_change_results(ctx):
    """The wavefront split (paths in flight) does not change any path."""
    import rendertoy_gb300 as rt
    sc = scenes.cornell_mixed()
    ctx.upload(sc)
    a = ctx.trace_paths(20, 16, 0, 3, 8, seed=1)
    ctx.set_option(rt.OPT_WAVE_PATHS, 97)
    try:
        b = ctx.trace_paths(20, 16, 0, 3, 8, seed=1)
        c = ctx.render_pt(20, 16, 3, 8, seed=1)
    finally:
        ctx.set_option(rt.OPT_WAVE_PATHS, 0)
    d = ctx.render_pt(20, 16, 3, 8, seed=1)
    assert np.array_equal(bits(a), bits(b))
    assert np.array_equal(bits(c), bits(d))


def test_ray_sort_does_not_change_results(ctx):
    """Sorting the extension queue by ray key (and the shading queue by
    material) only changes the order in which paths are visited: per-path
    radiance and the accumulated image stay bit-identical."""
    import rendertoy_gb300 as rt
    sc = scenes.displaced_icosphere(subdiv=3)
    ctx.upload(sc)
    a = ctx.trace_paths(40, 30, 0, 3, 12, seed=5)
    c = ctx.render_pt(64, 48, 6, 12, seed=5)
    for opts in ((rt.OPT_SORT_RAYS,), (rt.OPT_SORT_RAYS, rt.OPT_SORT_MATERIAL)):
        for o in opts:
            ctx.set_option(o, 1)
        try:
            b = ctx.trace_paths(40, 30, 0, 3, 12, seed=5)
            d = ctx.render_pt(64, 48, 6, 12, seed=5)
        finally:
            for o in opts:
                ctx.set_option(o, 0)
        assert np.array_equal(bits(a), bits(b)), opts
        assert np.array_equal(bits(c), bits(d)), opts


def test_edge_cases(ctx, oracle):
    import rendertoy_gb300 as rt
    # no emitters: no light samples are drawn; only the environment lights
    sc = scenes.cornell_box()
    sc.mats[:, 3:6] = 0
    sc.sky[:] = (0.5, 0.6, 0.7)
    sc.ground[:] = (0.2, 0.1, 0.0)
    ctx.upload(sc)
    assert len(ctx.emitters()) == 0
    got = ctx.trace_paths(8, 8, 0, 2, 5, seed=4)
    ref = oracle.scene(sc).trace_paths(8, 8, 0, 2, 5, 4)
    assert rel_close(got, ref, 1e-4, 1e-6).all(-1).mean() >= 0.99
    # 1 x 1 image, max depth 1
    ctx.upload(scenes.cornell_box())
    one = ctx.render_pt(1, 1, 3, 1, seed=0)
    assert one.shape == (1, 1, 3)
    # empty scene: every ray misses and sees the environment
    sc0 = scenes.cornell_box()
    sc0.verts = sc0.verts[:0]
    sc0.norms = sc0.norms[:0]
    sc0.tri_mesh = sc0.tri_mesh[:0]
    sc0.sky[:] = (1.0, 2.0, 3.0)
    ctx.upload(sc0)
    tri, _ = ctx.primary(4, 4)
    assert (tri == -1).all()
    img = ctx.render_pt(4, 4, 2, 5)
    assert np.isfinite(img).all()
    # invalid arguments return errors, not crashes
    ctx.upload(scenes.cornell_box())
    with pytest.raises(rt.RtxError):
        ctx.render_pt(0, 4, 1, 5)
    with pytest.raises(rt.RtxError):
        ctx.render_pt(4, 4, 1, 0)
    bad = scenes.cornell_box()
    bad.tri_mesh = bad.tri_mesh.copy()
    bad.tri_mesh[3] = 99
    with pytest.raises(rt.RtxError):
        ctx.upload(bad)


@pytest.mark.gpu
def test_traversal_variants_agree(ctx):
    """The binary batch walk (0), the binary while-while walk with ray refill
    (1) and the 4-wide tree (2, the default) find the same closest hits and
    occluders (nearest triangle, lower-id ties): per-path radiance is
    bit-identical."""
    import rendertoy_gb300 as rt
    ctx.upload(scenes.cornell_mixed())
    out = {}
    try:
        for trav in (0, 1, 2):
            ctx.set_option(rt.OPT_TRAVERSAL, trav)
            out[trav] = ctx.trace_paths(40, 32, 0, 2, 8, seed=3)
    finally:
        ctx.set_option(rt.OPT_TRAVERSAL, 2)
    for trav in (1, 2):
        assert np.array_equal(np.nan_to_num(out[trav], nan=-7).view(np.uint32),
                              np.nan_to_num(out[0], nan=-7).view(np.uint32)), trav


def test_progressive_checkpoint_resume(ctx):
    """A frame rendered in chunks of samples, checkpointed to the host after
    each chunk and resumed in a fresh context, equals the frame rendered in
    one call bit for bit (also when each chunk runs in several waves)."""
    import rendertoy_gb300 as rt
    from helpers import same_bits
    sc = scenes.cornell_mixed()
    ctx.upload(sc)
    W, H, spp, depth, seed = 40, 30, 16, 8, 77
    whole = ctx.render_pt(W, H, spp, depth, seed=seed)
    chunks = [(0, 5), (5, 6), (11, 5)]
    img = None
    for k, (first, n) in enumerate(chunks):
        with rt.Context(0) as other:  # a new process would do the same
            other.upload(sc)
            if k == 1:
                other.set_option(rt.OPT_WAVE_PATHS, 777)
            buf = np.zeros((H, W, 3), np.float32) if img is None else img.copy()  # the checkpoint
            img = other.render_pt_progressive(W, H, first, n, spp, depth, seed=seed, out=buf)
    assert same_bits(img, whole)
    with pytest.raises(rt.RtxError):
        ctx.render_pt_progressive(W, H, 10, 7, spp, depth)  # past the frame's samples


def test_lobe_variants_agree(ctx):
    """The shading kernel leaves out the refraction and clearcoat lobes when
    no material of the scene uses them (spec_trans / clearcoat all zero).
    The same scene with one more, unused material that has both lobes runs
    the full kernel: single renders, per-path traces and textured batch
    frames are bit-identical between the two."""
    import dataclasses

    from helpers import same_bits
    extra = scenes.material((0.5, 0.5, 0.5), spec_trans=1.0, clearcoat=1.0)[None]
    cases = [scenes.cornell_box(), scenes.displaced_icosphere(subdiv=3),
             scenes.procedural_scene(3, n_tris=5000)[0]]
    try:
        for sc in cases:
            full = dataclasses.replace(sc, mats=np.vstack([sc.mats, extra]).astype(np.float32))
            out = []
            for s in (sc, full):
                ctx.upload(s)
                out.append((ctx.trace_paths(40, 30, 0, 3, 12, seed=9), ctx.render_pt(48, 40, 4, 12, seed=9)))
            for x, y in zip(*out):
                assert same_bits(x, y), sc.name
    finally:
        ctx.upload(scenes.cornell_box())


def test_sorts_auto_by_scene():
    """RTX_OPT_SORT_RAYS defaults to 2 (sort when the scene has 4,096
    triangles or more) and RTX_OPT_SORT_MATERIAL to 2 (sort when a material
    refracts or there are 8 or more); small, large and many-material scenes
    render the same bits with either option at 0, 1 and 2."""
    import rendertoy_gb300 as rt
    from helpers import same_bits
    with rt.Context(0) as c:
        assert c.get_option(rt.OPT_SORT_RAYS) == 2
        assert c.get_option(rt.OPT_SORT_MATERIAL) == 2
        for sc in (scenes.cornell_box(), scenes.displaced_icosphere(subdiv=4), scenes.cornell_mixed()):
            c.upload(sc)
            ref = c.render_pt(48, 40, 4, 8, seed=3)
            for opt in (rt.OPT_SORT_RAYS, rt.OPT_SORT_MATERIAL):
                for v in (0, 1, 2):
                    c.set_option(opt, v)
                    assert same_bits(ref, c.render_pt(48, 40, 4, 8, seed=3)), (sc.name, opt, v)
                c.set_option(opt, 2)


def test_nonfinite_triangles_are_never_hit():
    """Triangles with non-finite vertices (NaN coordinates, infinities,
    coordinates whose box centre overflows) are accepted and never hit: the
    Cornell box renders the same bits with six such triangles appended as a
    mesh of its own with a non-emitting material."""
    import rendertoy_gb300 as rt
    from helpers import same_bits
    sc = scenes.cornell_box()
    bad = np.array([[np.nan] * 9,
                    [0, 0, 0, 10, 0, 0, np.nan, 5, 5],
                    [3e38] * 9,
                    [-3e38, 2e38, 1, -3e38, 2e38, 2, -3e38, 2e38, 3],
                    [np.inf, 0, 0, 0, 10, 0, 0, 0, 10],
                    [0, -np.inf, 0, 10, 0, 0, 0, 0, 10]], np.float32)
    plain_mat = int(np.nonzero(np.all(sc.mats[:, 3:6] == 0, axis=1))[0][0])
    sc2 = scenes.Scene(verts=np.concatenate([sc.verts, bad]),
                       norms=np.concatenate([sc.norms, np.zeros_like(bad)]),
                       tri_mesh=np.concatenate([sc.tri_mesh, np.full(len(bad), len(sc.mesh_mat), np.int32)]),
                       mesh_mat=np.append(sc.mesh_mat, plain_mat).astype(np.int32),
                       mesh_smooth=np.append(sc.mesh_smooth, 0).astype(np.uint8),
                       mats=sc.mats, sky=sc.sky, ground=sc.ground, camera=sc.camera, name="cornell+nonfinite")
    with rt.Context(0) as c:
        c.upload(sc)
        ref = c.render_pt(48, 40, 4, 8, seed=3)
        c.upload(sc2)
        got = c.render_pt(48, 40, 4, 8, seed=3)
    assert np.isfinite(ref).all()
    assert same_bits(ref, got)


def test_absorbing_media(ctx, oracle):
    """Beer-Lambert absorption inside refracting materials (extinction != 1,
    RenderToy's renderer.cpp:293, 311, 319): per-path radiance against the oracle
    in the mixed-lobe room with its glass made absorbing."""
    sc = scenes.cornell_mixed()
    glass = sc.mats[:, 15] > 0  # spec_trans: the refracting materials
    assert glass.any()
    sc.mats[glass, 17] = 80.0                       # at_distance
    sc.mats[glass, 18:21] = (0.35, 0.6, 0.85)       # extinction per channel
    ctx.upload(sc)
    got = ctx.trace_paths(24, 20, 0, 4, 10, seed=7)
    ref = oracle.scene(sc).trace_paths(24, 20, 0, 4, 10, 7)
    close = rel_close(got, ref, 1e-4, 1e-6).all(-1)
    assert close.mean() >= 0.99, close.mean()
    # the absorption actually entered some paths: their radiance differs
    # from the same room without it
    sc2 = scenes.cornell_mixed()
    ctx.upload(sc2)
    plain = ctx.trace_paths(24, 20, 0, 4, 10, seed=7)
    assert (np.abs(plain - got) > 1e-6).any()
