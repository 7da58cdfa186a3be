"""The host BVH builder (rendertoy_gb300/csrc/bvh_build.cpp) on its own, no GPU.

tests/bvh_check.cpp is compiled with the builder's source and run on seeded
triangle sets: the displaced icosphere at subdivision 7 (327,680 triangles,
enough for the builder to use threads and to cut its first passes into
chunks), random and clustered triangles, a flat plane (one axis without
extent), many copies of one triangle (all centroids equal) and triangles
with non-finite vertices.  For each set and leaf size it builds with 1, 3
and 8 threads and checks that every thread count gives the same bits, that
both trees (binary and 4-wide) hold every triangle exactly once, and that
every child box contains its subtree's vertices.  It first checks the host
thread pool the builder uses (every index once; a worker's exception reaches
the caller).  The GPU tests cover what the kernels do with the trees.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from rendertoy_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "rendertoy_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    from rendertoy_gb300 import build
    exe = str(tmp_path_factory.mktemp("bvh") / "bvh_check")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(build.CUDA_HOME, "include"),
           "-I" + CSRC, os.path.join(ROOT, "tests", "bvh_check.cpp"), os.path.join(CSRC, "bvh_build.cpp"),
           "-o", exe, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def triangle_sets():
    rng = np.random.RandomState(11)
    sets = {"icosphere7": scenes.displaced_icosphere(subdiv=7).verts,
            "random": rng.rand(3000, 9),
            "clustered": np.repeat(rng.rand(20, 9), 500, axis=0) + rng.rand(10000, 9) * 1e-6,
            "same": np.tile(rng.rand(1, 9), (2000, 1))}
    flat = rng.rand(5000, 9)
    flat[:, [2, 5, 8]] = 0.25
    sets["flat"] = flat
    bad = rng.rand(4000, 9)
    bad[7, 3] = np.nan                 # one NaN coordinate
    bad[100, :] = np.nan               # every vertex NaN
    bad[200, 0] = np.inf
    bad[300, 4] = -np.inf
    bad[400, :] = 3e38                 # finite, but its box centre overflows
    bad[500, [0, 3, 6]] = -3e38
    sets["nonfinite"] = bad
    return {k: (np.asarray(v, np.float32) + np.float32(0.0)).astype(np.float32) for k, v in sets.items()}


@pytest.mark.parametrize("leaf", [1, 4, 8])
def test_builder_threads_agree_and_trees_hold_every_triangle(checker, tmp_path, leaf):
    for name, verts in triangle_sets().items():
        path = tmp_path / f"{name}.f32"
        verts.tofile(path)
        r = subprocess.run([checker, str(path), str(leaf)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (name, leaf, r.stdout, r.stderr)
