#!/usr/bin/env python3
"""bench.py — path-tracing throughput of librtx on GB300.

Workload (one step = one frame): the seeded displaced icosphere (20 * 4^8 =
1,310,720 triangles, Perlin displacement 0.05 r) in the Cornell room,
1024 x 1024 pixels, 64 samples per pixel, max depth 12, then the Compositor's
Gaussian blur (sigma 8, size 49) and a 5 x 5 edge-detect convolution of the
result.  Metric: Msamples/s (pixel samples per second), with Mrays/s beside it.

  value : device time of the step with the scene and image resident in HBM
          (CUDA events on the library's stream, L2 flushed between steps);
  e2e   : the same step through the C ABI with host (pinned) buffers: the image
          is copied back after the render and each filter copies its image in
          and out, as RenderToy's Image does; host wall clock.
  roofline : the closest-hit traversal kernel (k_extend), algorithmic bytes =
          BVH nodes visited x node size (112 B for the default 4-wide tree,
          64 B binary) + triangles tested x 48 B + 52 B of ray I/O per ray,
          counted by an instrumented (untimed) run of the same step, against
          the measured HBM copy bandwidth and (roofline.l2) against the L2
          read bandwidth this run measures (the tree and triangles, 112 MB,
          stay L2-resident).  roofline_connect: the same for the occlusion
          kernel (80 B of shadow-record I/O per ray).  roofline_shade: the
          shading kernel, the largest of the frame, against SM instruction
          issue (4 warp instructions per SM per clock at the sampled SM clock)
          and FP32 (128 lanes per SM per clock); its executed instructions per
          sample come from an ncu capture (profiles/k_shade_issue.txt).
  c1     : the 36-triangle Cornell box (256^2, 16 spp, depth 8), which is
          cache-resident and so reported as SM issue utilisation and active
          lanes per warp (instructions per frame from an ncu capture,
          profiles/cornell_c1_issue.txt), not as a memory fraction.
  batched : 16 procedural scenes traced through one wavefront per frame,
          autotuned and replayed as a CUDA graph (the batched workload on
          fewer scenes, so that the run stays within minutes).
  cpu_baseline : the oracle's restatement of RenderToy's renderer (octree +
          priority-queue traversal) on the host cores, on a bounded sample, at
          the workload's depth 12 and at RenderToy's native depth 5, with the
          restatement's measured speed relative to RenderToy's own build
          (oracle/cpu_calibration.json, made where RenderToy's sources are).
  denoiser : the learned denoiser outside the timed frames: one Adam step on a
          32 x 256^2 minibatch and one 1920 x 1088 inference, device time and
          tensor-core TFLOP/s against the measured BF16 peak.
  compositor : each filter timed alone on the resident image, achieved GB/s of
          its algorithmic bytes as a fraction of the measured HBM bandwidth.
  obj_import : the host OBJ importer (one thread) on 262,144 triangles of the
          bench mesh written as OBJ text; config.scene_upload_s is the whole
          upload of the bench scene (threaded BVH build, device copies).

``--impl reference`` times RenderToy's CPU path on the same workload (its
compiled sources where they run here, otherwise the oracle restatement).
Multi-GPU: each rank renders its own frame (no collective on the data path);
scaling is weak.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RES = 1024
SPP = 64
DEPTH = 12
SUBDIV = 8
BLUR_SIZE, BLUR_SIGMA = 49, 8.0
EDGE5 = np.array([[0, 0, -1, 0, 0], [0, -1, -2, -1, 0], [-1, -2, 16, -2, -1],
                  [0, -1, -2, -1, 0], [0, 0, -1, 0, 0]], np.float32)
WORKLOAD = (f"displaced icosphere ({20 * 4 ** SUBDIV} tris, subdiv {SUBDIV}, Perlin 0.05r, seed 1) "
            f"in the Cornell room; {RES}x{RES}, {SPP} spp, max depth {DEPTH}; "
            f"Gaussian blur sigma {BLUR_SIGMA} size {BLUR_SIZE} + 5x5 edge convolution")


def peaks(key="hbm_gbs"):
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d[key]), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}[key], "fallback"


def denoiser_block(ctx, rank):
    """The learned denoiser on the tensor cores: one Adam step on a 32 x 256^2
    minibatch (forward + backward + update; the training config's minibatch)
    and inference on a 1920 x 1088 frame, each timed with the library's CUDA
    events (median of 10 after 3 warm-up runs).  Tensor work = the padded
    convolutions the kernels execute: 2 * 9 * Cin * Cout per pixel of each
    layer's resolution, x 3 for a training step (forward, data and weight
    gradients)."""
    import torch
    ctx.dn_init(rank)
    fwd = sum(2 * 9 * L["cin_pad"] * L["cout_pad"] / 4 ** L["level"] for L in ctx.dn_layers())
    g = torch.Generator(device="cuda").manual_seed(rank)
    N, H, W = 32, 256, 256
    raw = torch.rand(N, H, W, 11, device="cuda", generator=g)
    raw[..., :3] *= 4.0
    raw[..., 10] = 4.0
    tgt = torch.rand(N, H, W, 3, device="cuda", generator=g)

    def med(fn, n=10):
        for _ in range(3):
            fn()
        t = []
        for _ in range(n):
            fn()
            t.append(ctx.stats()["last_gpu_ms"])
        return float(np.median(t))

    train_ms = med(lambda: ctx.dn_train_step(raw, tgt, lr=3e-4))
    train_launches = ctx.stats()["kernel_launches"]
    fr = torch.rand(1, 1088, 1920, 11, device="cuda", generator=g)
    fr[..., 10] = 4.0
    out = torch.empty(1, 1088, 1920, 3, device="cuda")
    infer_ms = med(lambda: ctx.dn_infer(fr, out))
    peak, kind = peaks("bf16_tflops")
    hbm, _ = peaks()
    train_tf = 3 * fwd * N * H * W / (train_ms * 1e-3) / 1e12
    infer_tf = fwd * 1088 * 1920 / (infer_ms * 1e-3) / 1e12
    bound_train = layer_bound_ms(ctx.dn_layers(), N * H * W, peak, hbm, train=True)
    bound_infer = layer_bound_ms(ctx.dn_layers(), 1088 * 1920, peak, hbm, train=False)
    return {"train_step_ms": train_ms, "minibatch": [N, H, W], "train_tflops": train_tf,
            "train_kernel_launches": train_launches, "infer_ms_1920x1088": infer_ms, "infer_tflops": infer_tf,
            "gflop_per_mpixel_forward": fwd * 1e6 / 1e9,
            "roofline": {"bound": "tensor", "achieved": train_tf, "peak": peak, "peak_kind": kind,
                         "unit": "TFLOP/s", "frac": train_tf / peak,
                         "note": "whole training step (all its launches) against the bf16 burst peak"},
            "layer_roofline": {"train_bound_ms": bound_train, "train_frac": bound_train / train_ms,
                               "infer_bound_ms": bound_infer, "infer_frac": bound_infer / infer_ms,
                               "note": "sum over layers and passes of max(FLOPs / bf16 peak, "
                                       "compulsory bytes / HBM peak) against the measured time"}}


def layer_bound_ms(layers, px0, tflops, gbs, train):
    """Lower bound on the network's time from each convolution's own
    roofline: per layer and pass, max(tensor FLOPs / peak, compulsory HBM
    bytes / peak), summed.  Compulsory bytes per output pixel of a layer
    (BF16 activations): forward reads its sources once (an upsampled source
    at a quarter of the pixels) and writes Cout; the data gradient reads dout
    and the source (ReLU mask) and writes the source's gradient; the weight
    gradient reads dout and the source.  The small elementwise kernels
    (pooling, loss, Adam) are left out, so the bound is optimistic."""
    t = 0.0
    for L in layers:
        px = px0 / 4 ** L["level"]
        ci, co = L["cin_pad"], L["cout_pad"]
        c1 = L["c1_pad"]
        src = (c1 / 4 if L["up1"] else c1) + (ci - c1)
        flops = 2 * 9 * ci * co * px
        passes = [(flops, (src + co) * 2 * px)]
        if train:
            passes += [(flops, (co + src + ci) * 2 * px), (flops, (co + src) * 2 * px)]
        t += sum(max(f / (tflops * 1e12), b / (gbs * 1e9)) for f, b in passes)
    return t * 1e3


def compositor_block(ctx, img, tmp, out, flush, sms, clk_mhz):
    """The Compositor filters timed alone on the resident 1024^2 image (the
    library's CUDA events around the whole call, median of 10; L2 flushed
    before each run): algorithmic bytes per pixel = 12 B read + 12 B written
    per pass (blur: two passes; 5 x 5 convolution: one; bloom: extract + blur
    x, then blur y + add = 12 + 12 + 24 + 12).  The filters keep the
    reference's unfused multiply-then-add per tap, so FP32 issue bounds them
    before HBM does: `bound_us` = max(bytes / HBM peak, FP32 operations /
    the FP32 rate), `frac_bound` = that bound / the measured time.  The
    kernels issue packed FP32 instructions (two lanes' worth of operations
    each), which halves their instruction count but not the FP32 pipe's
    work: the rate is 128 lane-operations per SM per clock, at the SM clock
    sampled during the run."""
    import torch
    peak, kind = peaks()

    def med(fn):
        t = []
        for _ in range(12):
            flush.zero_()
            torch.cuda.synchronize()
            fn()
            t.append(ctx.stats()["last_gpu_ms"])
        return float(np.median(t[2:]))

    import rendertoy_gb300 as rt
    px = RES * RES
    fp32_ops = sms * 128 * clk_mhz * 1e6  # FP32 lane-operations per second
    res = {}
    for fma in (0, 1):
        ctx.set_option(rt.OPT_COMPOSITOR_FMA, fma)
        per_tap = 1 if fma else 2  # fused multiply-add, or a multiply and an add
        blur_ops = 2 * BLUR_SIZE * 3 * per_tap  # two passes, per tap and channel
        for name, fn, bpp, ops in (
                ("gaussian_blur_49", lambda: ctx.gaussian_blur(img, BLUR_SIZE, BLUR_SIGMA, out=tmp), 48, blur_ops),
                ("convolve_5x5", lambda: ctx.convolve(tmp, EDGE5, absval=True, out=out), 24, 25 * 3 * per_tap + 3),
                ("bloom_49", lambda: ctx.bloom(img, BLUR_SIZE, BLUR_SIGMA, 1.0, out=tmp), 60, blur_ops + 8)):
            ms = med(fn)
            gbs = bpp * px / (ms * 1e-3) / 1e9
            bound_us = max(bpp * px / (peak * 1e9), ops * px / fp32_ops) * 1e6
            res[name + ("_fma" if fma else "")] = {
                "ms": ms, "bytes_per_pixel": bpp, "achieved_gbs": gbs, "frac_hbm": gbs / peak,
                "fp32_ops_per_pixel": ops, "bound_us": bound_us, "frac_bound": bound_us / (ms * 1e3)}
    ctx.set_option(rt.OPT_COMPOSITOR_FMA, 0)
    res["peak_gbs"] = peak
    res["peak_kind"] = kind
    res["note"] = ("default entries: RenderToy's rounding (bit-exact); *_fma: RTX_OPT_COMPOSITOR_FMA, each tap's "
                   "multiply-add fused (within 1e-5 of the taps' magnitude)")
    return res


def profile_facts(name):
    """The `key value` lines of a profiles/ summary (ncu-derived constants)."""
    p = os.path.join(ROOT, "profiles", name)
    d = {}
    if os.path.exists(p):
        for ln in open(p):
            f = ln.split()
            if len(f) >= 2 and not ln.startswith("#"):
                try:
                    d[f[0]] = float(f[1])
                except ValueError:
                    pass
    return d


def l2_probe(ctx):
    """Read bandwidth of a plain streaming kernel (rtx_probe_read_bandwidth,
    16-byte ld.global.cg loads, L2-only caching) over buffers that fit the L2
    (32 and 64 MiB), one the size of the traversal working set (112 MiB:
    4-wide nodes + triangles of the bench scene) and one far beyond it (4 GiB,
    HBM), each read many times in one launch after an untimed pass.  The L2
    peak is the larger of the two L2-resident figures."""
    res = {}
    for mib, passes in ((32, 4000), (64, 2000), (112, 1000), (4096, 12)):
        res[f"{mib}MiB"] = ctx.probe_read_bandwidth(mib << 20, passes)
    return {"peak_gbs": max(res["32MiB"], res["64MiB"]), "probe_gbs": res,
            "how": "rtx_probe_read_bandwidth: grid-stride 16-byte ld.global.cg reads, 8 blocks x 256 "
                   "threads per SM, repeated passes in one launch, CUDA events"}


def traversal_roofline(bytes_frame, launches_frame, ms_frame, hbm, hbm_kind, l2):
    """Algorithmic bytes per launch / average launch time, against HBM and L2."""
    per_launch = bytes_frame / launches_frame
    avg_ms = ms_frame / launches_frame
    ach = per_launch / (avg_ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": ach, "peak": hbm, "peak_kind": hbm_kind, "unit": "GB/s",
            "frac": ach / hbm, "bytes_per_launch": per_launch, "avg_launch_ms": avg_ms,
            "l2": {"achieved": ach, "peak": l2["peak_gbs"], "peak_kind": "measured in this run (L2 probe)",
                   "unit": "GB/s", "frac": ach / l2["peak_gbs"]}}


def c1_block(local, sms, clk_mhz, reps=10):
    """The Cornell box (36 triangles, 256^2, 16 spp, depth 8).  The whole
    scene sits in L1/L2, so the frame is bound by instruction issue and lane
    divergence: SM issue utilisation = warp instructions per frame / (SMs x 4
    issue slots x SM clock x frame time), active lanes per warp = thread
    instructions / warp instructions.  Instructions per frame come from an
    ncu capture of the same frame (profiles/cornell_c1_issue.txt; the counts
    are fixed by the seed), the frame time from CUDA events here (median)."""
    import rendertoy_gb300 as rt
    from rendertoy_gb300 import scenes
    W = H = 256
    spp, depth = 16, 8
    with rt.Context(local) as c:
        c.upload(scenes.cornell_box())
        import torch
        out = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
        for i in range(3):
            c.render_pt(W, H, spp, depth, seed=1 + i, out=out)
        ms = []
        for i in range(reps):
            c.render_pt(W, H, spp, depth, seed=1, out=out)
            ms.append(c.stats()["last_gpu_ms"])
        launches = c.stats()["kernel_launches"]
    med = float(np.median(ms))
    res = {"workload": "Cornell box (36 triangles), 256x256, 16 spp, max depth 8, seed 1",
           "ms_per_frame": med, "msamples_per_s": W * H * spp / (med / 1e3) / 1e6,
           "kernel_launches": launches, "l2": "scene resident in L1/L2 (not flushed)"}
    f = profile_facts("cornell_c1_issue.txt")
    if "warp_inst_per_frame" in f:
        res["issue_utilisation"] = f["warp_inst_per_frame"] / (sms * 4 * clk_mhz * 1e6 * med / 1e3)
        res["active_lanes_per_warp_inst"] = f["thread_inst_per_frame"] / f["warp_inst_per_frame"]
        res["warp_inst_per_frame"] = f["warp_inst_per_frame"]
        res["source"] = "profiles/cornell_c1_issue.txt (ncu instruction counts) / this run's frame time"
    return res


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x, ws, device="cuda"):
    """Max over ranks of a per-rank timing (the only collective: control plane)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, slowest_seconds, ws):
    """Whole-job throughput: every rank processes its own units (weak scaling),
    the job takes as long as the slowest rank."""
    return units_per_rank * ws / slowest_seconds


def cpu_calibration():
    """The restatement's speed relative to RenderToy's own build on the same
    work, measured where RenderToy's sources are (oracle/calibrate_cpu.py)."""
    p = os.path.join(ROOT, "oracle", "cpu_calibration.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return {"restatement_over_reference_speed": {k: d[k]["speedup"] for k in ("paths_d12", "paths_d5",
                                                                            "render_d5") if k in d},
            "measured_on": d.get("machine"), "source": "oracle/cpu_calibration.json"}


def cpu_sample_rate(sc, seconds=12.0, threads=0, kind="oracle", depth=DEPTH):
    """Msamples/s of RenderToy's CPU path (restated) on a bounded sample of
    the workload: random pixels of the 1024^2 film, 1 sample each, at the
    given max depth (the workload's 12, or RenderToy's native 5)."""
    from oracle import bind
    if kind == "reference":
        chk = bind.load("ref")
    else:
        bind.build()
        chk = bind.load("oracle")
    s = chk.scene(sc)
    rng = np.random.RandomState(0)
    n = 256
    total_samples, total_t = 0, 0.0
    while True:
        pix = rng.choice(RES * RES, n, replace=False).astype(np.int32)
        t0 = time.perf_counter()
        s.trace_paths(RES, RES, 0, 1, depth, 1, pixels=pix, threads=threads)
        dt = time.perf_counter() - t0
        total_samples += n
        total_t += dt
        if total_t >= seconds:
            break
        left = seconds - total_t
        n = int(min(max(n * 2, n * left / max(dt, 1e-3)), 200000))
    cores = threads or os.cpu_count()
    return total_samples / total_t / 1e6, total_samples, total_t, cores


BATCH_DEPTH = 8


def obj_import_block(sc, n_tris=262144):
    """Host OBJ import (rtx_obj_import through rendertoy_gb300.ObjModel,
    arrays copied out included): the first `n_tris` triangles of the bench
    mesh written as OBJ text (`v` / `vn` per corner, `f v//vn`, one object),
    parsed on one host thread.  Written outside the timing, median of 3."""
    import tempfile

    import rendertoy_gb300 as rt
    n = min(n_tris, sc.n_tris)
    d = tempfile.mkdtemp()
    path = os.path.join(d, "mesh.obj")
    with open(path, "w") as f:
        f.write("o mesh\n")
        np.savetxt(f, sc.verts[:n].reshape(-1, 3), fmt="v %.6f %.6f %.6f")
        np.savetxt(f, sc.norms[:n].reshape(-1, 3), fmt="vn %.6f %.6f %.6f")
        k = np.arange(1, 3 * n + 1).reshape(-1, 3)
        np.savetxt(f, np.repeat(k, 2, axis=1), fmt="f %d//%d %d//%d %d//%d")
    size = os.path.getsize(path)
    ts = []
    for _ in range(3):
        t = time.perf_counter()
        m = rt.ObjModel(path)
        ts.append(time.perf_counter() - t)
    assert len(m.tri_mesh) == n
    os.remove(path)
    os.rmdir(d)
    sec = float(np.median(ts))
    return {"triangles": n, "bytes": size, "ms": sec * 1e3, "mb_per_s": size / sec / 1e6,
            "mtris_per_s": n / sec / 1e6, "threads": 1}


def run_batched(local, rank, n_scenes, steps, warmup, ws=1):
    """The batched config: seeded procedural scenes (1e3-2e6 triangles each,
    textures, 1-4 blackbody quad lights), each frame at its own resolution
    (256^2 .. 1920 x 1080) and spp (1..64), max depth 8, all traced through one
    wavefront per step (rtx_render_batch), captured as a CUDA graph after the
    autotuner picked block size and wave capacity on a reduced-spp copy of the
    frame.  Step = one batch frame; value = samples / device time."""
    import torch
    import rendertoy_gb300 as rt
    from rendertoy_gb300 import scenes
    t0 = time.perf_counter()
    scs, jobs = [], []
    for k in range(n_scenes):
        sc, job = scenes.procedural_scene(1000 * rank + k)
        scs.append(sc)
        jobs.append(dict(scene=k, W=job["W"], H=job["H"], spp=job["spp"], seed=k + 1))
    gen_s = time.perf_counter() - t0
    with rt.Context(local) as ctx:
        t0 = time.perf_counter()
        ctx.batch_upload(scs)
        upload_s = time.perf_counter() - t0
        tris = sum(sc.n_tris for sc in scs)
        pix = sum(j["W"] * j["H"] for j in jobs)
        samples = sum(j["W"] * j["H"] * j["spp"] for j in jobs)
        small = [dict(j, spp=max(1, j["spp"] // 8)) for j in jobs]
        tune = ctx.batch_autotune(small, BATCH_DEPTH)
        ctx.set_option(rt.OPT_GRAPH, 1)
        out = torch.empty(pix * 3, dtype=torch.float32, device="cuda")
        for i in range(warmup):
            ctx.render_batch([dict(j, seed=j["seed"] + 1000 * i) for j in jobs], BATCH_DEPTH, out=out)
        ctx.synchronize()
        ms = []
        with Clocks(local) as clk:
            for i in range(steps):
                ctx.render_batch([dict(j, seed=j["seed"] + 7919 * (i + 1)) for j in jobs], BATCH_DEPTH, out=out)
                ms.append(ctx.stats()["last_gpu_ms"])
    total_ms = reduce_max(sum(ms), ws)
    value = job_rate(samples * steps, total_ms / 1e3, ws) / 1e6
    config = {"workload": f"{n_scenes} procedural scenes in one batch frame, max depth {BATCH_DEPTH}",
              "triangles": tris, "pixels": pix, "samples_per_frame": samples,
              "resolutions": sorted({f"{j['W']}x{j['H']}" for j in jobs}),
              "spp_range": [min(j["spp"] for j in jobs), max(j["spp"] for j in jobs)],
              "scene_gen_s": round(gen_s, 1), "upload_and_bvh_s": round(upload_s, 1),
              "l2": "frame data far larger than L2"}
    return value, total_ms / steps, config, tune, clk.summary()


def batched(args, ws, rank, local):
    value, ms, config, tune, clocks = run_batched(local, rank, args.scenes, args.steps, args.warmup, ws)
    if rank == 0:
        line = {
            "metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scenes; no dataset)",
            "config": config, "autotune": tune, "graph": True, "clocks": clocks,
        }
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--subdiv", type=int, default=SUBDIV)
    ap.add_argument("--profile", action="store_true",
                    help="render one step of the workload and exit (for ncu)")
    ap.add_argument("--res", type=int, default=RES, help="with --profile: film size")
    ap.add_argument("--spp", type=int, default=SPP, help="with --profile: samples per pixel")
    ap.add_argument("--depth", type=int, default=DEPTH, help="with --profile: max path depth")
    ap.add_argument("--scene", default="icosphere", choices=["icosphere", "cornell"],
                    help="with --profile: the scene rendered (cornell: the 36-triangle Cornell box, no filters)")
    ap.add_argument("--workload", default="icosphere", choices=["icosphere", "batched"],
                    help="batched: 64 procedural scenes in one wavefront per frame (not the default)")
    ap.add_argument("--scenes", type=int, default=64, help="with --workload batched")
    ap.add_argument("--opt", action="append", default=[],
                    help="library option NAME=VALUE for the run (e.g. sort_rays=1), recorded in config")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    from rendertoy_gb300 import scenes

    if args.impl == "reference":
        if rank != 0:
            return
        sc = scenes.displaced_icosphere(subdiv=args.subdiv)
        kind = "oracle"
        try:
            from oracle import bind
            bind.load("ref")
            kind = "reference"
        except OSError:
            kind = "oracle"
        except FileNotFoundError:
            kind = "oracle"
        per_step = max(args.cpu_seconds / max(args.steps, 1), 2.0)
        vals = []
        for _ in range(args.warmup and 1):
            cpu_sample_rate(sc, seconds=1.0, kind=kind)
        tot_s, tot_t = 0, 0.0
        for _ in range(args.steps):
            v, ns, t, cores = cpu_sample_rate(sc, seconds=per_step, kind=kind)
            vals.append(v)
            tot_s += ns
            tot_t += t
        value = tot_s / tot_t / 1e6
        line = {"impl": "reference", "metric": "Msamples/s", "value": value, "unit": "Msamples/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": tot_t / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "sample": "random pixels of the film, 1 spp each"},
                "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": cores,
                                 "kind": "reference" if kind == "reference" else "port",
                                 "sample": f"{tot_s} samples (random pixels x 1 spp, depth {DEPTH}) "
                                           f"in {tot_t:.1f} s",
                                 "calibration": cpu_calibration()},
                "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    import __graft_entry__ as ge
    ge.build()
    import rendertoy_gb300 as rt

    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if args.workload == "batched":
        return batched(args, ws, rank, local)

    t0 = time.perf_counter()
    sc = scenes.cornell_box() if (args.profile and args.scene == "cornell") else \
        scenes.displaced_icosphere(subdiv=args.subdiv)
    gen_s = time.perf_counter() - t0
    ctx = rt.Context(local)
    opts = {}
    for o in args.opt:
        k, v = o.split("=")
        ctx.set_option(getattr(rt, "OPT_" + k.upper()), int(v))
        opts[k] = int(v)
    t0 = time.perf_counter()
    ctx.upload(sc)
    upload_s = time.perf_counter() - t0
    st0 = ctx.stats()
    if args.profile:
        out = torch.empty((args.res, args.res, 3), dtype=torch.float32, device="cuda")
        ctx.render_pt(args.res, args.res, args.spp, args.depth, seed=1, out=out)
        st = ctx.stats()
        if args.scene == "icosphere":
            tmp = torch.empty_like(out)
            ctx.gaussian_blur(out, BLUR_SIZE, BLUR_SIGMA, out=tmp)
            ctx.convolve(tmp, EDGE5, absval=True, out=out)
        ctx.synchronize()
        print(json.dumps({"profile": True, "scene": args.scene, "res": args.res, "spp": args.spp,
                          "depth": args.depth, **st}))
        return
    stream = torch.cuda.ExternalStream(ctx.stream)
    dev = torch.device("cuda", local)
    img = torch.empty((RES, RES, 3), dtype=torch.float32, device=dev)
    blur = torch.empty_like(img)
    edge = torch.empty_like(img)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    seed = 1 + rank

    def step(i):
        ctx.render_pt(RES, RES, SPP, DEPTH, seed=seed + 1000 * i, out=img)
        ctx.gaussian_blur(img, BLUR_SIZE, BLUR_SIGMA, out=blur)
        ctx.convolve(blur, EDGE5, absval=True, out=edge)

    ctx.set_option(rt.OPT_ASYNC, 1)
    ctx.set_option(rt.OPT_KERNEL_TIMING, 1)
    for i in range(args.warmup):
        step(i)
    ctx.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    step_ms, rays_e, rays_s = [], 0, 0
    kt = {k: 0.0 for k in ("extend_ms", "shade_ms", "connect_ms", "extend_launches", "shade_launches",
                           "connect_launches")}
    with Clocks(local) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            ctx.render_pt(RES, RES, SPP, DEPTH, seed=seed + 1000 * i, out=img)
            ctx.gaussian_blur(img, BLUR_SIZE, BLUR_SIGMA, out=blur)
            ctx.convolve(blur, EDGE5, absval=True, out=edge)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            # the filters leave the render's timers and ray counters untouched
            s = ctx.stats()
            for k in kt:
                kt[k] += s[k]
            rays_e += s["extension_rays"]
            rays_s += s["shadow_rays"]
    total_ms = reduce_max(sum(step_ms), ws)
    samples = RES * RES * SPP * args.steps
    value = job_rate(samples, total_ms / 1e3, ws) / 1e6
    mrays = (rays_e + rays_s) * ws / (total_ms / 1e3) / 1e6

    clocks = clk.summary()
    clk_mhz = clocks["sm_mhz"] or 2070.0  # unsampled: the GB300's maximum SM clock

    # Per-kernel launch times for the rooflines come from frames with the
    # occlusion launches serialised (RTX_OPT_OVERLAP = 0): in the timed frames
    # above a vertex's occlusion launch shares the GPU with the next vertex's
    # closest-hit launch, so each one's event-to-event time includes the other.
    kt_overlapped = kt
    serial_frames = max(1, min(args.steps, 5))
    kt = {k: 0.0 for k in kt_overlapped}
    serial_ms = []
    ctx.set_option(rt.OPT_OVERLAP, 0)
    for i in range(serial_frames):
        flush.zero_()
        torch.cuda.synchronize()
        ctx.render_pt(RES, RES, SPP, DEPTH, seed=seed + 1000 * i, out=img)
        ctx.synchronize()
        s = ctx.stats()
        serial_ms.append(s["last_gpu_ms"])
        for k in kt:
            kt[k] += s[k] * args.steps / serial_frames  # scaled to the timed frames' count
    ctx.set_option(rt.OPT_OVERLAP, 1)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count

    # instrumented run (untimed): node visits and triangle tests per frame
    ctx.set_option(rt.OPT_COUNT_VISITS, 1)
    ctx.set_option(rt.OPT_KERNEL_TIMING, 0)
    ctx.render_pt(RES, RES, SPP, DEPTH, seed=seed, out=img)
    cs = ctx.stats()
    ctx.set_option(rt.OPT_COUNT_VISITS, 0)
    # kernels per step: the render's launches + blur (2) + convolution (1)
    launches = (cs["kernel_launches"] + 3) * args.steps
    frames = args.steps
    per_frame = {k: v / frames for k, v in kt.items()}
    ext_bytes_frame = (cs["ext_node_visits"] * cs["node_bytes"] + cs["ext_tri_tests"] * 48 +
                       cs["extension_rays"] * 52)
    con_bytes_frame = (cs["shadow_node_visits"] * cs["node_bytes"] + cs["shadow_tri_tests"] * 48 +
                       cs["shadow_rays"] * 80)
    peak, peak_kind = peaks()
    l2 = l2_probe(ctx)
    roof = traversal_roofline(ext_bytes_frame, per_frame["extend_launches"], per_frame["extend_ms"], peak,
                              peak_kind, l2)
    roof_con = traversal_roofline(con_bytes_frame, per_frame["connect_launches"], per_frame["connect_ms"],
                                  peak, peak_kind, l2)
    # DRAM bytes per launch from the ncu capture in profiles/ (fixed + per-ray
    # fit, cold L2 per launch), scaled to this run's rays per launch
    traffic = None
    fit = profile_facts("k_extend_traffic.txt")
    if "dram_bytes_per_extension_ray" in fit:
        traffic = (fit.get("dram_bytes_per_launch_fixed", 0.0) +
                   fit["dram_bytes_per_extension_ray"] * cs["extension_rays"] / per_frame["extend_launches"])
    roof.update({"kernel": "k_extend", "traffic": traffic,
                 "launch_times": f"{serial_frames} frames with the occlusion launches serialised "
                                 "(RTX_OPT_OVERLAP=0); the timed frames overlap them",
                 "overlapped_avg_launch_ms": kt_overlapped["extend_ms"] / kt_overlapped["extend_launches"],
                 "extend_share_of_step": kt["extend_ms"] / sum(step_ms),
                 "per_extension_ray": {"node_visits": cs["ext_node_visits"] / cs["extension_rays"],
                                       "tri_tests": cs["ext_tri_tests"] / cs["extension_rays"]}})
    roof_con.update({"kernel": "k_connect", "traffic": None,
                     "overlapped_avg_launch_ms": kt_overlapped["connect_ms"] / kt_overlapped["connect_launches"],
                     "connect_share_of_step": kt["connect_ms"] / sum(step_ms),
                     "per_shadow_ray": {"node_visits": cs["shadow_node_visits"] / cs["shadow_rays"],
                                        "tri_tests": cs["shadow_tri_tests"] / cs["shadow_rays"]}})
    # shading: issue- and FP32-bound; instructions per sample from ncu
    shade = {"kernel": "k_shade", "bound": "issue", "shade_share_of_step": kt["shade_ms"] / sum(step_ms),
             "avg_launch_ms": per_frame["shade_ms"] / per_frame["shade_launches"],
             "sm_mhz": clk_mhz, "sms": sms}
    sf = profile_facts("k_shade_issue.txt")
    if "warp_inst_per_sample" in sf:
        spf = RES * RES * SPP
        t = per_frame["shade_ms"] / 1e3
        issue_peak = sms * 4 * clk_mhz * 1e6  # warp instructions per second
        fp32_peak = sms * 128 * clk_mhz * 1e6  # FP32 lane-operations per second
        ach_issue = sf["warp_inst_per_sample"] * spf / t
        ach_fp32 = sf["fp32_ops_per_sample"] * spf / t
        shade.update({"achieved": ach_issue / 1e9, "peak": issue_peak / 1e9, "unit": "G warp inst/s",
                      "frac": ach_issue / issue_peak, "peak_kind": "4 issue slots x SMs x sampled SM clock",
                      "fp32": {"achieved": ach_fp32 / 1e12, "peak": fp32_peak / 1e12, "unit": "T lane-ops/s",
                               "frac": ach_fp32 / fp32_peak},
                      "active_lanes_per_warp_inst": sf.get("active_lanes_per_warp_inst"),
                      "source": "profiles/k_shade_issue.txt (ncu instructions per sample) / this run's "
                                "k_shade time"})

    # end to end through the C ABI with pinned host buffers
    ctx.set_option(rt.OPT_ASYNC, 0)
    h_img = torch.empty((RES, RES, 3), dtype=torch.float32, pin_memory=True)
    h_blur = torch.empty_like(h_img, pin_memory=True)
    h_edge = torch.empty_like(h_img, pin_memory=True)
    e2e_steps = max(1, args.steps)
    ctx.render_pt(RES, RES, SPP, DEPTH, seed=seed, out=h_img)
    if ws > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        ctx.render_pt(RES, RES, SPP, DEPTH, seed=seed + 1000 * i, out=h_img)
        ctx.gaussian_blur(h_img, BLUR_SIZE, BLUR_SIGMA, out=h_blur)
        ctx.convolve(h_blur, EDGE5, absval=True, out=h_edge)
    e2e_s = reduce_max(time.perf_counter() - t0, ws)
    img_bytes = RES * RES * 12
    e2e = {"value": RES * RES * SPP * e2e_steps * ws / e2e_s / 1e6, "unit": "Msamples/s",
           "h2d_bytes_per_step": 2 * img_bytes + 84 + BLUR_SIZE * 4 + 25 * 4,
           "d2h_bytes_per_step": 3 * img_bytes, "steps": e2e_steps}

    comp = compositor_block(ctx, img, blur, edge, flush, sms, clk_mhz)
    dn = denoiser_block(ctx, rank)
    c1 = c1_block(local, sms, clk_mhz)
    bval, bms, bconf, btune, bclk = run_batched(local, rank, 16, 2, 1)
    batch = {"value": bval, "unit": "Msamples/s", "ms_per_frame": bms, "steps": 2, "warmup": 1,
             "config": bconf, "autotune": btune, "clocks": bclk, "graph": True}

    cpu = None
    obj = obj_import_block(sc) if rank == 0 else None
    if rank == 0:
        v, ns, t, cores = cpu_sample_rate(sc, seconds=args.cpu_seconds)
        v5, ns5, t5, _ = cpu_sample_rate(sc, seconds=max(2.0, args.cpu_seconds / 3), depth=5)
        cpu = {"value": v, "unit": "Msamples/s", "cores": cores, "kind": "port",
               "sample": f"{ns} samples (random pixels of the 1024^2 film x 1 spp, depth {DEPTH}) "
                         f"in {t:.1f} s; octree build excluded",
               "depth5": {"value": v5, "sample": f"{ns5} samples at RenderToy's native depth 5 in {t5:.1f} s"},
               "calibration": cpu_calibration()}

    if rank == 0:
        line = {
            "metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene; no dataset)",
            "config": {"workload": WORKLOAD, "resolution": [RES, RES], "spp": SPP,
                       "max_depth": DEPTH, "triangles": sc.n_tris,
                       "l2": "flushed between steps (256 MiB write, outside the timed events)",
                       "bvh_build_ms": st0["bvh_build_ms"], "bvh_nodes": st0["bvh_nodes"],
                       "scene_upload_s": round(upload_s, 3), "scene_gen_s": round(gen_s, 2),
                       "options": opts},
            "obj_import": obj,
            "mrays_per_s": mrays,
            "overlap": {"step_ms": total_ms / args.steps,
                        "render_ms_serialised": float(np.median(serial_ms)),
                        "note": "RTX_OPT_OVERLAP: each vertex's occlusion launch on a second stream beside "
                                "the next vertex's closest-hit launch (timed frames); serialised for comparison"},
            "rays_per_step": {"extension": rays_e / args.steps, "shadow": rays_s / args.steps},
            "e2e": e2e,
            "roofline": roof,
            "roofline_connect": roof_con,
            "roofline_shade": shade,
            "l2_probe": l2,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": launches,
            "c1": c1,
            "batched": batch,
            "denoiser": dn,
            "compositor": comp,
        }
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
