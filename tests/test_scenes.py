"""Synthetic workload generators (sizes and emitter order)."""
import numpy as np

from rendertoy_gb300 import scenes


def test_cornell_box_counts():
    sc = scenes.cornell_box()
    assert sc.n_tris == 36  # 10 wall + 24 box + 2 light triangles
    assert list(sc.emitters()) == [34, 35]
    assert sc.mats.shape[1] == 24
    # 40 degree vertical field of view: top = tan(20 deg)
    top = (sc.camera[18] * 25.4 / 2) / sc.camera[16]
    assert abs(top - np.tan(np.radians(20))) < 1e-6


def test_icosphere_counts():
    v, f = scenes.icosphere(3)
    assert len(f) == 20 * 4 ** 3
    assert len(v) == 10 * 4 ** 3 + 2
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0)


def test_displaced_icosphere_small():
    sc = scenes.displaced_icosphere(subdiv=2)
    assert sc.n_tris == 12 + 20 * 4 ** 2
    assert sc.mesh_smooth.sum() == 1
    assert np.isfinite(sc.verts).all()


def test_perlin_range():
    p = np.random.RandomState(0).uniform(-10, 10, (10000, 3))
    n = scenes.perlin3(p, 1)
    assert np.abs(n).max() <= 1.1 and np.abs(n).mean() > 0.05
