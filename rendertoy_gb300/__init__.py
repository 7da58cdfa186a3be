"""rendertoy_gb300 — GB300 (sm_103a) implementation of RenderToy's path-tracing
hot path behind a C ABI (include/rtx.h, librtx.so).

This module is a thin ctypes binding of that ABI for Python callers (tests,
benchmarks): ``Context`` mirrors RenderToy's RenderContext / renderers /
Image filters.  Arrays may be numpy arrays (host) or any object exposing
``data_ptr()`` for device memory (e.g. a CUDA torch tensor); the library
detects which.  There is no CPU fallback: if librtx.so is missing or no GPU is
present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librtx.so")

OPT_ASYNC, OPT_WAVE_PATHS, OPT_BLOCK, OPT_SORT_MATERIAL, OPT_COUNT_VISITS, OPT_LEAF_SIZE, \
    OPT_PRIMARY_CACHE, OPT_KERNEL_TIMING, OPT_ACCUMULATE, OPT_TRAVERSAL, OPT_MIN_BUSY = \
    1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11

STATUS = {0: "RTX_OK", 1: "RTX_ERR_INVALID", 2: "RTX_ERR_CUDA", 3: "RTX_ERR_NOMEM",
          4: "RTX_ERR_NO_SCENE", 5: "RTX_ERR_DEVICE"}

# every entry point include/rtx.h declares
EXPORTS = [
    "rtx_create", "rtx_destroy", "rtx_last_error", "rtx_version", "rtx_set_option",
    "rtx_get_option", "rtx_get_stream", "rtx_set_stream", "rtx_synchronize", "rtx_get_stats",
    "rtx_scene_upload", "rtx_scene_emitters", "rtx_scene_set_emitters", "rtx_render_pt", "rtx_trace_paths",
    "rtx_render_aov", "rtx_primary_hits", "rtx_intersect", "rtx_image_convolve",
    "rtx_image_gaussian_blur", "rtx_image_edge_detect", "rtx_image_bloom",
    "rtx_image_gaussian_blur_noalloc", "rtx_nn_gemm_bf16",
]


class RtxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Stats(C.Structure):
    _fields_ = [("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("ext_node_visits", C.c_uint64), ("ext_tri_tests", C.c_uint64),
                ("shadow_node_visits", C.c_uint64), ("shadow_tri_tests", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("extend_launches", C.c_uint64),
                ("last_gpu_ms", C.c_double), ("extend_ms", C.c_double), ("shade_ms", C.c_double),
                ("connect_ms", C.c_double), ("bvh_build_ms", C.c_double), ("bvh_nodes", C.c_int32), ("bvh_leaves", C.c_int32),
                ("bvh_depth", C.c_int32), ("node_bytes", C.c_int32), ("tri_bytes", C.c_int32),
                ("reserved", C.c_int32), ("ext_rays_by_depth", C.c_uint64 * 16)]


_lib = None


def lib() -> C.CDLL:
    """Load librtx.so (built by rendertoy_gb300.build); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError(f"{LIB_PATH} is not built: run python -m rendertoy_gb300.build")
    L = C.CDLL(LIB_PATH)
    vp, i, f, u64 = C.c_void_p, C.c_int, C.c_float, C.c_uint64
    sig = {
        "rtx_create": (i, [C.POINTER(vp), i]),
        "rtx_destroy": (None, [vp]),
        "rtx_last_error": (C.c_char_p, [vp]),
        "rtx_version": (i, []),
        "rtx_set_option": (i, [vp, i, C.c_int64]),
        "rtx_get_option": (i, [vp, i, C.POINTER(C.c_int64)]),
        "rtx_get_stream": (vp, [vp]),
        "rtx_set_stream": (i, [vp, vp]),
        "rtx_synchronize": (i, [vp]),
        "rtx_get_stats": (i, [vp, C.POINTER(Stats)]),
        "rtx_scene_upload": (i, [vp, i, vp, vp, vp, i, vp, vp, i, vp, vp, vp]),
        "rtx_scene_emitters": (i, [vp, vp, i, C.POINTER(i)]),
        "rtx_scene_set_emitters": (i, [vp, vp, i]),
        "rtx_render_pt": (i, [vp, vp, i, i, i, i, u64, vp]),
        "rtx_trace_paths": (i, [vp, vp, i, i, i, i, i, u64, vp]),
        "rtx_render_aov": (i, [vp, vp, i, i, f, f, vp, vp, vp]),
        "rtx_primary_hits": (i, [vp, vp, i, i, vp, vp]),
        "rtx_intersect": (i, [vp, i, vp, vp, vp, vp]),
        "rtx_image_convolve": (i, [vp, vp, vp, i, i, vp, i, i, i, i, i]),
        "rtx_image_gaussian_blur": (i, [vp, vp, vp, i, i, i, f]),
        "rtx_image_edge_detect": (i, [vp, vp, vp, i, i]),
        "rtx_image_bloom": (i, [vp, vp, vp, i, i, i, f, f]),
        "rtx_image_gaussian_blur_noalloc": (i, [vp, vp, i, i, i, f, vp, C.c_char_p, C.c_size_t]),
        "rtx_nn_gemm_bf16": (i, [vp, i, i, i, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a):
    """Address of a numpy array (host) or a device tensor (data_ptr())."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


class Context:
    """An rtx_context: one GPU, one stream, one uploaded scene."""

    def __init__(self, device: int = 0):
        self.L = lib()
        h = C.c_void_p()
        r = self.L.rtx_create(C.byref(h), device)
        if r != 0:
            raise RtxError(r, "rtx_create failed (is a CUDA device present?)")
        self.h = h
        self.scene = None

    def _check(self, r):
        if r != 0:
            raise RtxError(r, self.L.rtx_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.rtx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- options / stream / stats -------------------------------------------
    def set_option(self, opt, value):
        self._check(self.L.rtx_set_option(self.h, opt, int(value)))

    def get_option(self, opt):
        v = C.c_int64()
        self._check(self.L.rtx_get_option(self.h, opt, C.byref(v)))
        return v.value

    @property
    def stream(self) -> int:
        return self.L.rtx_get_stream(self.h) or 0

    def synchronize(self):
        self._check(self.L.rtx_synchronize(self.h))

    def stats(self) -> dict:
        s = Stats()
        self._check(self.L.rtx_get_stats(self.h, C.byref(s)))
        d = {k: getattr(s, k) for k, _ in Stats._fields_ if k not in ("reserved", "ext_rays_by_depth")}
        d["ext_rays_by_depth"] = list(s.ext_rays_by_depth)
        return d

    # -- scene ---------------------------------------------------------------
    def upload(self, sc):
        keep = [_f32(sc.verts), _f32(sc.norms), np.ascontiguousarray(sc.tri_mesh, np.int32),
                np.ascontiguousarray(sc.mesh_mat, np.int32),
                np.ascontiguousarray(sc.mesh_smooth, np.uint8), _f32(sc.mats), _f32(sc.sky),
                _f32(sc.ground)]
        v, n, tm, mm, ms, mats, sky, gr = keep
        self._check(self.L.rtx_scene_upload(self.h, sc.n_tris, _ptr(v), _ptr(n), _ptr(tm),
                                            len(mm), _ptr(mm), _ptr(ms), len(mats), _ptr(mats),
                                            _ptr(sky), _ptr(gr)))
        self.scene = sc

    def emitters(self):
        n = C.c_int()
        self._check(self.L.rtx_scene_emitters(self.h, None, 0, C.byref(n)))
        out = np.zeros(max(n.value, 1), np.int32)
        self._check(self.L.rtx_scene_emitters(self.h, _ptr(out), len(out), C.byref(n)))
        return out[:n.value]

    def set_emitters(self, ids):
        ids = np.ascontiguousarray(ids, np.int32)
        self._check(self.L.rtx_scene_set_emitters(self.h, _ptr(ids), len(ids)))

    def _cam(self, camera):
        return _f32(self.scene.camera if camera is None else camera)

    # -- renderers ------------------------------------------------------------
    def render_pt(self, W, H, spp, max_depth, seed=0, camera=None, out=None):
        cam = self._cam(camera)
        o = np.zeros((H, W, 3), np.float32) if out is None else out
        self._check(self.L.rtx_render_pt(self.h, _ptr(cam), W, H, spp, max_depth, seed, _ptr(o)))
        return o

    def trace_paths(self, W, H, first_sample, n_samples, max_depth, seed=0, camera=None, out=None):
        cam = self._cam(camera)
        o = np.zeros((n_samples, H * W, 3), np.float32) if out is None else out
        self._check(self.L.rtx_trace_paths(self.h, _ptr(cam), W, H, first_sample, n_samples,
                                           max_depth, seed, _ptr(o)))
        return o

    def aov(self, W, H, near, far, camera=None):
        cam = self._cam(camera)
        n = np.zeros((H, W, 3), np.float32)
        a = np.zeros((H, W, 3), np.float32)
        d = np.zeros((H, W, 3), np.float32)
        self._check(self.L.rtx_render_aov(self.h, _ptr(cam), W, H, near, far, _ptr(n), _ptr(a),
                                          _ptr(d)))
        return n, a, d

    def primary(self, W, H, camera=None):
        cam = self._cam(camera)
        tri = np.zeros((H, W), np.int32)
        tuv = np.zeros((H, W, 3), np.float32)
        self._check(self.L.rtx_primary_hits(self.h, _ptr(cam), W, H, _ptr(tri), _ptr(tuv)))
        return tri, tuv

    def intersect(self, rays, exclude=None):
        rays = _f32(rays).reshape(-1, 6)
        n = len(rays)
        ex = None if exclude is None else np.ascontiguousarray(exclude, np.int32)
        tri = np.zeros(n, np.int32)
        tuv = np.zeros((n, 3), np.float32)
        self._check(self.L.rtx_intersect(self.h, n, _ptr(rays), _ptr(ex), _ptr(tri), _ptr(tuv)))
        return tri, tuv

    # -- denoiser building blocks ---------------------------------------------
    def gemm_bf16(self, A, B, out=None):
        """C = A @ B.T on the tensor cores; A, B are uint16 arrays of BF16 bits
        (or device tensors of dtype bfloat16)."""
        M, K = A.shape
        N = B.shape[0]
        C_ = np.zeros((M, N), np.float32) if out is None else out
        self._check(self.L.rtx_nn_gemm_bf16(self.h, M, N, K, _ptr(A), _ptr(B), _ptr(C_)))
        return C_

    # -- compositor -------------------------------------------------------------
    @staticmethod
    def _img_io(img, out):
        if hasattr(img, "data_ptr"):
            H, W = int(img.shape[0]), int(img.shape[1])
            return img, out, W, H
        img = _f32(img)
        H, W = img.shape[:2]
        return img, (np.zeros_like(img) if out is None else out), W, H

    def convolve(self, img, kernel, normalize=False, length=False, absval=False, out=None):
        img, out, W, H = self._img_io(img, out)
        k = _f32(kernel)
        self._check(self.L.rtx_image_convolve(self.h, _ptr(img), _ptr(out), W, H, _ptr(k),
                                              k.shape[0], k.shape[1], int(normalize), int(length),
                                              int(absval)))
        return out

    def gaussian_blur(self, img, size, sigma, out=None):
        img, out, W, H = self._img_io(img, out)
        self._check(self.L.rtx_image_gaussian_blur(self.h, _ptr(img), _ptr(out), W, H, size, sigma))
        return out

    def edge_detect(self, img, out=None):
        img, out, W, H = self._img_io(img, out)
        self._check(self.L.rtx_image_edge_detect(self.h, _ptr(img), _ptr(out), W, H))
        return out

    def bloom(self, img, size, sigma, threshold, out=None):
        img, out, W, H = self._img_io(img, out)
        self._check(self.L.rtx_image_bloom(self.h, _ptr(img), _ptr(out), W, H, size, sigma,
                                           threshold))
        return out
