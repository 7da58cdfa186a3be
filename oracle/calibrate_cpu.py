"""Speed of the oracle restatement against RenderToy's own compiled renderer
(TEST INFRASTRUCTURE: measurement only).

The timed CPU baseline on the GPU host is the restatement (oracle/rt_oracle.cpp):
RenderToy's sources are not present there.  This script, run where they are
(``make -C oracle ref`` built oracle/_ref/), times both on the same work and
writes oracle/cpu_calibration.json, which the benchmark reports beside its CPU
number:

* ``paths_d12`` / ``paths_d5``: the same random pixels x 1 sample of the
  displaced-icosphere workload (1,310,732 triangles, 1024^2 film), per-path
  drivers of both (the reference's PathTracingRenderer::Radiance with the
  recursion cap patched to depth 12, resp. the unmodified cap of 5 vertices);
* ``render_d5``: RenderToy's own PathTracingRenderer::Render (unmodified, its
  OpenMP loop and shared buffer) on a 32 x 32 film x 16 spp at its native
  depth 5, against the restatement rendering the same film.  Render()
  parallelises over samples (src/renderer.cpp:247), so spp is kept at or above
  the thread count.

speedup = restatement samples/s / reference samples/s (> 1: the restatement
is faster, so a GPU-over-restatement ratio understates GPU-over-reference).

    python oracle/calibrate_cpu.py [--seconds S] [--threads T]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from oracle import bind  # noqa: E402
from rendertoy_gb300 import scenes  # noqa: E402

RES = 1024


def _rate(fn, n_first, seconds):
    """Samples/s of fn(n) (n samples per call), growing n until `seconds`."""
    n, done, spent = n_first, 0, 0.0
    while spent < seconds:
        t0 = time.perf_counter()
        fn(n)
        dt = time.perf_counter() - t0
        done += n
        spent += dt
        n = int(min(max(n * 2, n * (seconds - spent) / max(dt, 1e-3)), 100000))
    return done / spent, done, spent


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seconds", type=float, default=10.0)
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args()
    bind.build(ref=True)
    orc, ref, ref_orig = bind.load("oracle"), bind.load("ref"), bind.load("ref_orig")
    sc = scenes.displaced_icosphere(subdiv=8)
    so, sr, sro = orc.scene(sc), ref.scene(sc), ref_orig.scene(sc)
    threads = args.threads or os.cpu_count()
    out = {"machine": {"arch": platform.machine(), "cpus": os.cpu_count(), "threads": threads},
           "workload": f"displaced icosphere ({sc.n_tris} triangles), {RES}^2 film"}
    for depth, rsc, tag in ((12, sr, "paths_d12"), (5, sro, "paths_d5")):
        rng = np.random.RandomState(depth)

        def run(s, n):
            pix = rng.choice(RES * RES, n, replace=False).astype(np.int32)
            s.trace_paths(RES, RES, 0, 1, depth, 1, pixels=pix, threads=threads)

        r_o, n_o, t_o = _rate(lambda n: run(so, n), 256, args.seconds)
        r_r, n_r, t_r = _rate(lambda n: run(rsc, n), 256, args.seconds)
        out[tag] = {"oracle_msamples_s": r_o / 1e6, "reference_msamples_s": r_r / 1e6,
                    "speedup": r_o / r_r, "oracle_samples": n_o, "reference_samples": n_r}
        print(tag, out[tag], flush=True)
    W = H = 32
    spp = max(16, threads)
    t0 = time.perf_counter()
    so.render_pt(W, H, spp, 5, 1, threads=threads)
    t_o = time.perf_counter() - t0
    _, t_r = sro.render_native(W, H, spp, 5, threads=threads)
    n = W * H * spp
    out["render_d5"] = {"film": [W, H], "spp": spp, "oracle_s": t_o, "reference_render_s": t_r,
                        "oracle_msamples_s": n / t_o / 1e6, "reference_msamples_s": n / t_r / 1e6,
                        "speedup": t_r / t_o}
    print("render_d5", out["render_d5"], flush=True)
    with open(os.path.join(HERE, "cpu_calibration.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
