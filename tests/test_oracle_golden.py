"""The oracle (oracle/rt_oracle.cpp) against the reference's own outputs.

The golden vectors in tests/golden were produced by RenderToy's own sources
(tests/golden/make_golden.py); the restatement must reproduce them bit for bit.
"""
import numpy as np
import pytest

from helpers import bits, scene_from_fixture


@pytest.mark.parametrize("tag", ["cornell", "mixed"])
def test_scene_primary_aov_paths(oracle, golden, tag):
    g = golden(f"scene_{tag}")
    sc = scene_from_fixture(g)
    s = oracle.scene(sc)
    W, H = int(g["W"]), int(g["H"])
    near, far = float(sc.camera[19]), float(sc.camera[20])
    assert np.array_equal(s.emitters(), g["emitters"])
    assert np.array_equal(sc.emitters(), g["emitters"])
    tri, tuv = s.primary(W, H)
    assert np.array_equal(tri, g["primary_tri"])
    assert np.array_equal(bits(tuv), bits(g["primary_tuv"]))
    n, a, d = s.aov(W, H, near, far)
    for got, key in ((n, "aov_normal"), (a, "aov_albedo"), (d, "aov_depth")):
        assert np.array_equal(bits(got), bits(g[key])), key
    for depth in (5, 8):
        p = s.trace_paths(W, H, 0, 2, depth, int(g["seed"]))
        assert np.array_equal(bits(p), bits(g[f"paths_d{depth}"])), depth


def test_intersect(oracle, golden):
    g = golden("intersect_mixed")
    from rendertoy_gb300 import scenes
    s = oracle.scene(scenes.cornell_mixed())
    tri, tuv = s.intersect(g["rays"], g["exclude"])
    assert np.array_equal(tri, g["tri"])
    assert np.array_equal(bits(tuv), bits(g["tuv"]))


def test_bsdf(oracle, golden):
    g = golden("bsdf")
    n = len(g["eta"])
    for i in range(0, n, 3):
        f, pdf = oracle.bsdf_eval(g["mats"][i], g["eta"][i], g["N"][i], g["V"][i], g["L"][i])
        assert np.array_equal(bits(f), bits(g["eval_f"][i])) and bits(pdf) == bits(g["eval_pdf"][i])
        ok, od, col, sp = oracle.bsdf_sample(g["mats"][i], g["eta"][i], g["N"][i], g["V"][i],
                                             int(g["seed"]), i, 3)
        assert ok == g["sample_ok"][i]
        assert np.array_equal(bits(od), bits(g["sample_dir"][i]))
        assert np.array_equal(bits(col), bits(g["sample_color"][i]))
        assert bits(sp) == bits(g["sample_pdf"][i])


def test_compositor(oracle, golden):
    g = golden("compositor")
    for tag in ("a", "b"):
        img = g[f"img_{tag}"]
        k5 = g[f"k5_{tag}"]
        got = {
            "blur7": oracle.gaussian_blur(img, 7, 1.5),
            "blur49": oracle.gaussian_blur(img, 49, 8.0),
            "edge": oracle.edge_detect(img),
            "bloom": oracle.bloom(img, 9, 2.0, 0.8),
        }
        for flags in ((0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0), (0, 1, 1)):
            got["conv5_" + "".join(map(str, flags))] = oracle.convolve(
                img, k5, normalize=flags[0], length=flags[1], absval=flags[2])
        for name, out in got.items():
            rows = g[f"rows_{name}_{tag}"]
            assert rows.sum() > 0
            assert np.array_equal(bits(out[rows]), bits(g[f"{name}_{tag}"][rows])), (tag, name)
    for size, sigma in ((3, 0.8), (7, 1.5), (49, 8.0), (9, 2.0)):
        assert np.array_equal(bits(oracle.gaussian_weights(size, sigma)), bits(g[f"gw_{size}"]))


def test_reference_unit_assertions(oracle):
    """The reference's own unit checks that touch this path
    (RenderToy tests/mathfunctests.cpp:241-259): the 3x3 Gaussian centre and
    the Sobel coefficients, restated on the oracle."""
    w = oracle.gaussian_weights(3, 0.8).astype(np.float64)
    assert abs(np.outer(w, w)[1, 1] - 0.2725) < 1e-3  # separable form of the 3x3 kernel
    img = np.zeros((5, 5, 3), np.float32)
    img[2, 3] = 1.0
    e = oracle.convolve(img, np.array([[-1, 0, 1], [-2, 0, 2], [-1, 0, 1]], np.float32))
    assert e[2, 2, 0] == 2.0 and e[1, 2, 0] == 1.0


def test_rng_stream(oracle, golden):
    g = golden("rng")
    for key, ref in g.items():
        _, seed, pixel, sample = key.split("_")
        got = oracle.rng_floats(int(seed), int(pixel), int(sample), len(ref))
        assert np.array_equal(bits(got), bits(ref)), key
    assert np.all(got >= 0) and np.all(got < 1)


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors published with Random123."""
    def philox(c, k):
        M = 0xFFFFFFFF
        k0, k1 = k
        for _ in range(10):
            p0 = 0xD2511F53 * c[0]
            p1 = 0xCD9E8D57 * c[2]
            c = [(p1 >> 32) ^ c[1] ^ k0, p1 & M, (p0 >> 32) ^ c[3] ^ k1, p0 & M]
            k0, k1 = (k0 + 0x9E3779B9) & M, (k1 + 0xBB67AE85) & M
        return c
    assert philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]


def test_oracle_rng_matches_philox(oracle):
    """Draw k of a path is word k & 3 of Philox(counter (k>>2, sample, pixel, 0))."""
    f = oracle.rng_floats(0, 0, 0, 4)
    words = [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert np.array_equal(f, np.array([(w >> 8) * 2.0 ** -24 for w in words], np.float32))
