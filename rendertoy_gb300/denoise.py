"""The learned denoiser's data, training and evaluation (host side).

Training pairs come from the renderer itself on procedural scenes
(``scenes.procedural_scene``): the input is a radiance render at some spp plus
the albedo, normal and depth passes of the same camera and that spp (11
channels), the target a high-spp render with an independent seed.  The pairs
stay on the device; minibatches of random crops are gathered there and stepped
through ``Context.dn_train_step`` (forward, backward and Adam on the tensor
cores).  The network predicts a 5 x 5 filter per pixel that is applied to the
input radiance, trained on the relative squared error (its minimiser over
noisy targets is their mean, so the 4,096-spp targets' noise averages out
instead of biasing the result).

``study`` measures the denoised form against the plain one at equal accuracy
on one scene: a high-spp FP32 reference rendered as two independent halves
(so that its own noise can be taken out of every error), plain renders at
growing spp, the denoised renders at growing input spp (render + passes +
network + bloom), their relMSE against the reference and their frame times;
a frame whose denoised relMSE exceeds that of the plain render of equal time
falls back to the plain render.

    python -m rendertoy_gb300.denoise train --scenes 4000 --steps 20000 --in-spp 4,8192 \
        --target-spp 4096 --out DIR
    python -m rendertoy_gb300.denoise study --params DIR/params.npy --out DIR
    python -m rendertoy_gb300.denoise step --batch 8 --steps 2   # profiling

``step`` runs Adam steps of the network on one seeded random minibatch
already on the device (no rendering), the unit the convolution profiles
capture.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import scenes

EPS = 1e-2  # relMSE = mean (x - ref)^2 / (ref^2 + EPS)


def relmse(x, ref, eps=EPS):
    """Mean over pixels and channels of (x - ref)^2 / (ref^2 + eps); NaN or
    infinite pixels are masked and counted."""
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    ok = np.isfinite(x).all(-1) & np.isfinite(ref).all(-1)
    e = ((x - ref) ** 2 / (ref ** 2 + eps))[ok]
    return float(e.mean()), int((~ok).sum())


def relmse_corrected(x, ref_a, ref_b, eps=EPS):
    """relMSE of x against ref = (ref_a + ref_b) / 2, two renders of the
    same frame with independent random streams, with the reference's own
    noise taken out: for x independent of the reference,
    E[(x - ref)^2] = E[(x - mean)^2] + Var(ref), and (ref_a - ref_b)^2 / 4 is
    an unbiased per-pixel estimate of Var(ref).  Returns (raw relMSE,
    corrected relMSE, the reference's own relMSE estimate, masked pixels);
    NaN or infinite pixels of any of the three are masked."""
    x = np.asarray(x, np.float64)
    a = np.asarray(ref_a, np.float64)
    b = np.asarray(ref_b, np.float64)
    ok = np.isfinite(x).all(-1) & np.isfinite(a).all(-1) & np.isfinite(b).all(-1)
    x, a, b = x[ok], a[ok], b[ok]
    ref = 0.5 * (a + b)
    den = ref ** 2 + eps
    raw = ((x - ref) ** 2 / den).mean()
    noise = ((a - b) ** 2 / 4.0 / den).mean()
    return float(raw), float(raw - noise), float(noise), int((~ok).sum())


def frame_passes(ctx, sc, W, H):
    """albedo, normal, depth passes of the scene's camera (H x W x 3 each)."""
    n, a, d = ctx.aov(W, H, float(sc.camera[19]), float(sc.camera[20]))
    return a, n, d


def network_input(rad, albedo, normal, depth, spp):
    """One frame's network input [H][W][11] from its passes (host arrays)."""
    spp_plane = np.full(rad.shape[:2] + (1,), float(spp), np.float32)
    return np.concatenate([rad, albedo, normal, depth[..., :1], spp_plane], -1).astype(np.float32)


def pair_spp(seed, in_spp):
    """The input spp of pair `seed`: in_spp itself, or for a range (lo, hi)
    a log-uniform draw (seeded by the scene) so that one network serves
    many noise levels."""
    if isinstance(in_spp, (tuple, list)):
        lo, hi = np.log(in_spp[0]), np.log(in_spp[1])
        return int(round(np.exp(np.random.RandomState(int(seed)).uniform(lo, hi))))
    return int(in_spp)


def make_pairs(ctx, seeds, W=256, H=256, in_spp=4, target_spp=1024, max_depth=8,
               tri_range=(1e3, 2e5), log=print, device=False):
    """Render (input, target) pairs of the procedural scenes `seeds`:
    X [n][H][W][11], Y [n][H][W][3] (numpy arrays, or device tensors with
    device=True: then nothing is copied to the host).  Scene generation for
    the next scene runs on a host thread while the GPU renders."""
    import concurrent.futures as cf
    import torch
    seeds = [int(s) for s in seeds]
    dev = torch.device("cuda")
    X = torch.empty((len(seeds), H, W, 11), dtype=torch.float32, device=dev)
    Y = torch.empty((len(seeds), H, W, 3), dtype=torch.float32, device=dev)
    img = [torch.empty((H, W, 3), dtype=torch.float32, device=dev) for _ in range(4)]
    t0 = time.time()
    spps = []
    with cf.ThreadPoolExecutor(1) as pool:
        nxt = pool.submit(scenes.procedural_scene, seeds[0], tri_range=tri_range) if seeds else None
        for i, s in enumerate(seeds):
            sc, _ = nxt.result()
            if i + 1 < len(seeds):
                nxt = pool.submit(scenes.procedural_scene, seeds[i + 1], tri_range=tri_range)
            ctx.upload(sc)
            spp = pair_spp(s, in_spp)
            spps.append(spp)
            rad, nrm, alb, dep = img
            ctx.render_pt(W, H, spp, max_depth, seed=2 * s + 1, out=rad)
            ctx.aov(W, H, float(sc.camera[19]), float(sc.camera[20]), out=(nrm, alb, dep))
            ctx.synchronize()
            X[i, ..., 0:3] = rad
            X[i, ..., 3:6] = alb
            X[i, ..., 6:9] = nrm
            X[i, ..., 9] = dep[..., 0]
            X[i, ..., 10] = float(spp)
            torch.cuda.current_stream().synchronize()  # before the next render reuses the buffers
            ctx.render_pt(W, H, target_spp, max_depth, seed=2 * s + 2, out=Y[i])
            if log and (i + 1) % max(1, len(seeds) // 8) == 0:
                log(f"  pairs {i + 1}/{len(seeds)}  {time.time() - t0:.1f} s")
    torch.cuda.synchronize()
    if device:
        return X, Y
    return X.cpu().numpy(), Y.cpu().numpy()


def train(ctx, X, Y, steps, batch=32, crop=256, lr=3e-4, seed=0, log_every=200, log=print, decay_from=1.0):
    """Adam steps on random crops of random pairs (device-resident data; X, Y
    numpy arrays or device tensors).  The learning rate drops to lr / 10 for
    the steps after `decay_from` x steps.  Returns the per-step minibatch
    losses and the mean step time (ms)."""
    import torch
    n, H, W = X.shape[:3]
    crop = min(crop, H, W) // 16 * 16
    Xd = X if hasattr(X, "data_ptr") else torch.from_numpy(X).cuda()
    Yd = Y if hasattr(Y, "data_ptr") else torch.from_numpy(Y).cuda()
    g = torch.Generator().manual_seed(seed)
    losses, ms = [], []
    for it in range(steps):
        idx = torch.randint(0, n, (batch,), generator=g).cuda()
        y0 = int(torch.randint(0, H - crop + 1, (1,), generator=g))
        x0 = int(torch.randint(0, W - crop + 1, (1,), generator=g))
        xb = Xd[idx, y0:y0 + crop, x0:x0 + crop].contiguous()
        yb = Yd[idx, y0:y0 + crop, x0:x0 + crop].contiguous()
        rate = lr if it < decay_from * steps else lr / 10
        losses.append(ctx.dn_train_step(xb, yb, lr=rate))
        ms.append(ctx.stats()["last_gpu_ms"])
        if log and (it + 1) % log_every == 0:
            log(f"  step {it + 1}/{steps}  loss {np.mean(losses[-log_every:]):.4f}  "
                f"{np.mean(ms[-log_every:]):.2f} ms/step")
    return np.asarray(losses), float(np.mean(ms[min(5, len(ms) - 1):]))


def _timed(ctx, fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, (time.perf_counter() - t0) * 1e3


def _time_to(points, target):
    """Frame time at which a (ms, relMSE) curve, measured at increasing time,
    first reaches `target`: log-log interpolation between the two measured
    points around it; None when no measured point reaches it."""
    for (t0, e0), (t1, e1) in zip(points, points[1:]):
        if e0 > target >= e1 and e1 > 0 and e0 > 0:
            f = (math.log(e0) - math.log(target)) / (math.log(e0) - math.log(e1))
            return float(math.exp(math.log(t0) + f * (math.log(t1) - math.log(t0))))
    if points and 0 < points[0][1] <= target:
        return float(points[0][0])
    return None


def study(ctx, sc, W, H, ref_spp=16384, max_depth=12,
          denoise_spp=(1, 4, 16, 64, 256, 1024, 2048, 4096, 8192),
          plain_spp=(1, 4, 16, 64, 256, 1024, 4096), reps=20,
          bloom=(49, 8.0, 1.0), target=1e-3, seed=1, log=print, cache=None):
    """Denoised vs plain at equal accuracy on one scene (see the module text).
    The reference is two renders of ref_spp / 2 samples with independent
    random streams; errors are reported raw and with the reference's own
    noise removed (relmse_corrected), and times to the target use the
    corrected errors.  Times are device-synchronised wall times of the whole
    frame, its buffers resident on the device (median of `reps` runs for
    frames under a second, of 3 above).  `cache` (a dict) keeps the reference
    and the plain sweep for later studies of other networks on the same
    scene and settings."""
    ctx.upload(sc)
    cache = {} if cache is None else cache
    half = ref_spp // 2
    if "ref" not in cache:
        t0 = time.time()
        cache["ref"] = (ctx.render_pt(W, H, half, max_depth, seed=10_000 + seed),
                        ctx.render_pt(W, H, half, max_depth, seed=20_000 + seed))
        log(f"  reference 2 x {half} spp: {time.time() - t0:.1f} s")
    ref_a, ref_b = cache["ref"]
    out = {"scene": sc.name, "W": W, "H": H, "ref_spp": 2 * half, "max_depth": max_depth, "eps": EPS,
           "target_relmse": target, "plain": [], "denoised": []}
    import torch
    dev = lambda: torch.empty((H, W, 3), dtype=torch.float32, device="cuda")  # noqa: E731
    img, rad, alb, nrm, dep, den, fin = (dev() for _ in range(7))
    near, far = float(sc.camera[19]), float(sc.camera[20])

    def timed_reps(fn):
        first = _timed(ctx, fn)[1]
        n = reps if first < 1000.0 else 3
        times = [first] + [_timed(ctx, fn)[1] for _ in range(n - 1)]
        return float(np.median(times)), float(np.percentile(times, 99))

    # plain: relMSE and frame time per spp (device-resident frame)
    if "plain" not in cache:
        plain = []
        for spp in plain_spp:
            ms, p99 = timed_reps(lambda: ctx.render_pt(W, H, spp, max_depth, seed=seed, out=img))
            raw, corr, noise, bad = relmse_corrected(img.cpu().numpy(), ref_a, ref_b)
            plain.append({"spp": spp, "ms": ms, "ms_p99": p99, "relmse_raw": raw, "relmse": corr, "nan_px": bad})
            log(f"  plain {spp:5d} spp  {ms:9.2f} ms  relMSE {corr:.3e} (raw {raw:.3e})")
        cache["plain"] = (plain, noise)
    out["plain"], out["ref_noise_relmse"] = cache["plain"]
    # plain relMSE ~ c / spp (Monte Carlo): fitted on the corrected errors
    p = out["plain"]
    fit = [q for q in p if q["spp"] >= 16 and q["relmse"] > 0]
    c = float(np.median([q["relmse"] * q["spp"] for q in fit]))
    ms_per_spp = float(np.median([q["ms"] / q["spp"] for q in fit]))
    out["plain_fit"] = {"c": c, "ms_per_spp": ms_per_spp}
    measured = _time_to([(q["ms"], q["relmse"]) for q in p], target)
    out["plain_time_to_target_ms"] = measured if measured is not None else c / target * ms_per_spp
    out["plain_time_to_target_from"] = "measured" if measured is not None else "fit c / spp"
    out["plain_spp_to_target"] = c / target
    # denoised: render + passes + network + bloom, per input spp
    for spp in denoise_spp:
        def frame():
            ctx.render_pt(W, H, spp, max_depth, seed=seed, out=rad)
            ctx.aov(W, H, near, far, out=(nrm, alb, dep))
            ctx.denoise(rad, alb, nrm, dep, spp, out=den)
            if bloom:
                ctx.bloom(den, *bloom, out=fin)
        t_med, t_99 = timed_reps(frame)
        raw, e_den, _, bad = relmse_corrected(den.cpu().numpy(), ref_a, ref_b)
        _, e_in, _, _ = relmse_corrected(rad.cpu().numpy(), ref_a, ref_b)
        # the plain render of equal time (the fitted curve)
        e_plain_equal = float(c / max(t_med / ms_per_spp, 1e-9))
        fallback = e_den > e_plain_equal
        out["denoised"].append({"spp": spp, "ms_p50": t_med, "ms_p99": t_99, "relmse": e_den,
                                "relmse_raw": raw, "relmse_input": e_in, "nan_px": bad,
                                "relmse_plain_equal_time": e_plain_equal, "fallback": bool(fallback)})
        log(f"  denoised {spp} spp  p50 {t_med:.2f} ms  relMSE {e_den:.3e} (input {e_in:.3e}, plain at equal "
            f"time {e_plain_equal:.3e}){'  -> fallback' if fallback else ''}")
    # the denoised form with its fallback: each frame is the better of the
    # denoised and the plain render of equal time
    d = out["denoised"]
    curve = [(q["ms_p50"], min(q["relmse"], q["relmse_plain_equal_time"])) for q in d]
    out["denoised_time_to_target_ms"] = _time_to(curve, target)
    if out["denoised_time_to_target_ms"]:
        out["speedup_time_to_target"] = out["plain_time_to_target_ms"] / out["denoised_time_to_target_ms"]
    best = min(d, key=lambda q: q["relmse"])
    out["denoised_best"] = best
    out["plain_time_to_best_denoised_ms"] = float(c / best["relmse"] * ms_per_spp) if best["relmse"] > 0 else None
    if out["plain_time_to_best_denoised_ms"]:
        out["speedup_at_best_denoised_accuracy"] = out["plain_time_to_best_denoised_ms"] / best["ms_p50"]
    return out


def _main():
    import rendertoy_gb300 as rt
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "study", "step", "full"],
                    help="full: render the pairs once, train one network per --subsets size on the first "
                         "that many scenes, and study each (one process: the pairs never leave the device)")
    ap.add_argument("--out", default="denoise_out")
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--subsets", default="", help="with full: scene counts to train on, e.g. 192,1000,4000")
    ap.add_argument("--res", type=int, default=256)
    ap.add_argument("--target-spp", type=int, default=4096)
    ap.add_argument("--in-spp", default="4,8192",
                    help="input samples per pixel of the training pairs: N, or LO,HI (log-uniform per pair)")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--decay-from", type=float, default=0.9)
    ap.add_argument("--params", default="")
    ap.add_argument("--study-res", default="1920x1080")
    ap.add_argument("--ref-spp", type=int, default=16384)
    ap.add_argument("--denoise-spp", default="1,4,16,64,256,1024,2048,4096,8192")
    a = ap.parse_args()
    ctx = rt.Context(0)
    ctx.dn_init(0)
    if a.params:
        ctx.dn_set_params(np.load(a.params))
    if a.cmd == "step":
        import torch
        g = torch.Generator(device="cuda").manual_seed(0)
        xb = torch.rand(a.batch, a.res, a.res, 11, device="cuda", generator=g)
        xb[..., 10] = 64.0
        yb = 2 * torch.rand(a.batch, a.res, a.res, 3, device="cuda", generator=g)
        ms = []
        for _ in range(a.steps):
            loss = ctx.dn_train_step(xb, yb, lr=a.lr)
            ms.append(ctx.stats()["last_gpu_ms"])
        print(json.dumps({"batch": a.batch, "res": a.res, "steps": a.steps, "loss": loss, "ms": ms}))
        return
    os.makedirs(a.out, exist_ok=True)
    in_spp = tuple(int(v) for v in a.in_spp.split(","))
    in_spp = in_spp[0] if len(in_spp) == 1 else in_spp
    W, H = (int(v) for v in a.study_res.split("x"))
    dspp = tuple(int(v) for v in a.denoise_spp.split(","))

    def run_train(X, Y, n, tag):
        ctx.dn_init(0)
        t0 = time.time()
        losses, ms = train(ctx, X[:n], Y[:n], a.steps, batch=a.batch, lr=a.lr, decay_from=a.decay_from)
        np.save(os.path.join(a.out, f"params{tag}.npy"), ctx.dn_get_params())
        res = {"scenes": n, "res": a.res, "in_spp": a.in_spp, "target_spp": a.target_spp, "steps": a.steps,
               "batch": a.batch, "lr": a.lr, "decay_from": a.decay_from, "train_s": time.time() - t0,
               "ms_per_step": ms, "loss_first100": float(losses[:100].mean()),
               "loss_last100": float(losses[-100:].mean()),
               "loss_curve": [float(losses[i:i + 500].mean()) for i in range(0, len(losses), 500)]}
        json.dump(res, open(os.path.join(a.out, f"train{tag}.json"), "w"), indent=1)
        print(json.dumps({k: v for k, v in res.items() if k != "loss_curve"}), flush=True)
        return res

    study_cache = {}
    icosphere = scenes.displaced_icosphere()

    def run_study(tag):
        res = study(ctx, icosphere, W, H, ref_spp=a.ref_spp, denoise_spp=dspp, cache=study_cache)
        json.dump(res, open(os.path.join(a.out, f"study{tag}.json"), "w"), indent=1)
        print(json.dumps({k: v for k, v in res.items() if k not in ("plain", "denoised")}), flush=True)
        return res

    if a.cmd in ("train", "full"):
        t0 = time.time()
        X, Y = make_pairs(ctx, range(a.scenes), W=a.res, H=a.res, in_spp=in_spp, target_spp=a.target_spp,
                          device=True)
        data = {"scenes": a.scenes, "data_s": time.time() - t0}
        json.dump(data, open(os.path.join(a.out, "data.json"), "w"))
        print(json.dumps(data), flush=True)
        subsets = [int(v) for v in a.subsets.split(",")] if (a.cmd == "full" and a.subsets) else [a.scenes]
        for n in subsets:
            tag = f"_{n}" if a.cmd == "full" else ""
            run_train(X, Y, n, tag)
            if a.cmd == "full":
                run_study(tag)
    else:
        run_study("")


if __name__ == "__main__":
    _main()
