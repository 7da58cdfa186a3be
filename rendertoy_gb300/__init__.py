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

OPT_GRAPH = 12
OPT_SORT_RAYS = 13
OPT_STACK_LIMIT = 14
OPT_COMPOSITOR_FMA = 15
OPT_OVERLAP = 16
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
    "rtx_render_aov", "rtx_primary_hits", "rtx_intersect", "rtx_bsdf_eval", "rtx_bsdf_sample",
    "rtx_render_pt_progressive",
    "rtx_probe_read_bandwidth", "rtx_selftest_wait_timeout", "rtx_image_convolve",
    "rtx_image_gaussian_blur", "rtx_image_edge_detect", "rtx_image_bloom",
    "rtx_image_gaussian_blur_noalloc", "rtx_nn_gemm_bf16", "rtx_nn_conv3x3_fwd",
    "rtx_nn_conv3x3_dgrad", "rtx_nn_conv3x3_wgrad", "rtx_dn_init", "rtx_dn_info", "rtx_dn_layer",
    "rtx_dn_get_params", "rtx_dn_set_params", "rtx_dn_get_grads", "rtx_dn_get_adam", "rtx_dn_set_adam",
    "rtx_dn_loss_grads", "rtx_dn_train_step", "rtx_dn_infer", "rtx_denoise",
    "rtx_scene_set_texture_table", "rtx_texture_sample", "rtx_render_pt_resolved", "rtx_image_resolve",
    "rtx_image_tonemap", "rtx_image_gamma", "rtx_encode_bmp", "rtx_encode_ppm",
    "rtx_obj_import", "rtx_obj_free", "rtx_obj_info", "rtx_obj_triangles", "rtx_obj_mesh", "rtx_obj_material",
    "rtx_batch_upload", "rtx_render_batch", "rtx_batch_autotune",
]


class SceneDesc(C.Structure):
    _fields_ = [("n_tris", C.c_int), ("verts", C.c_void_p), ("norms", C.c_void_p), ("tri_mesh", C.c_void_p),
                ("n_meshes", C.c_int), ("mesh_mat", C.c_void_p), ("mesh_smooth", C.c_void_p),
                ("n_materials", C.c_int), ("materials", C.c_void_p), ("sky", C.c_void_p), ("ground", C.c_void_p),
                ("emitters", C.c_void_p), ("n_emitters", C.c_int)]


class Job(C.Structure):
    _fields_ = [("scene", C.c_int), ("camera", C.c_float * 21), ("W", C.c_int), ("H", C.c_int),
                ("spp", C.c_int), ("seed", C.c_uint64)]


class TuneResult(C.Structure):
    _fields_ = [("block", C.c_int64), ("wave_paths", C.c_int64), ("leaf_size", C.c_int64), ("ms", C.c_double),
                ("ms_default", C.c_double), ("trials", C.c_int), ("sort_material", C.c_int),
                ("traversal", C.c_int), ("sort_rays", C.c_int), ("overlap", C.c_int)]


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
                ("reserved", C.c_int32), ("ext_rays_by_depth", C.c_uint64 * 16),
                ("shade_launches", C.c_uint64), ("connect_launches", C.c_uint64)]


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
        "rtx_render_pt_progressive": (i, [vp, vp, i, i, i, i, i, i, u64, vp]),
        "rtx_render_aov": (i, [vp, vp, i, i, f, f, vp, vp, vp]),
        "rtx_primary_hits": (i, [vp, vp, i, i, vp, vp]),
        "rtx_intersect": (i, [vp, i, vp, vp, vp, vp]),
        "rtx_bsdf_eval": (i, [vp, i, vp, vp, vp, vp, vp, vp, vp]),
        "rtx_bsdf_sample": (i, [vp, i, vp, vp, vp, vp, u64, i, vp, vp, vp, vp]),
        "rtx_probe_read_bandwidth": (i, [vp, C.c_size_t, i, C.POINTER(C.c_double)]),
        "rtx_selftest_wait_timeout": (i, [vp, i]),
        "rtx_image_convolve": (i, [vp, vp, vp, i, i, vp, i, i, i, i, i]),
        "rtx_image_gaussian_blur": (i, [vp, vp, vp, i, i, i, f]),
        "rtx_image_edge_detect": (i, [vp, vp, vp, i, i]),
        "rtx_image_bloom": (i, [vp, vp, vp, i, i, i, f, f]),
        "rtx_image_gaussian_blur_noalloc": (i, [vp, vp, i, i, i, f, vp, C.c_char_p, C.c_size_t]),
        "rtx_nn_gemm_bf16": (i, [vp, i, i, i, vp, vp, vp, i, i]),
        "rtx_nn_conv3x3_fwd": (i, [vp, i, i, i, vp, i, i, vp, i, vp, vp, i, i, vp]),
        "rtx_nn_conv3x3_dgrad": (i, [vp, i, i, i, vp, i, vp, vp, i, i, vp, i, i, vp]),
        "rtx_nn_conv3x3_wgrad": (i, [vp, i, i, i, vp, i, vp, i, i, vp, i, vp]),
        "rtx_dn_init": (i, [vp, u64]),
        "rtx_dn_info": (i, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(i), C.POINTER(i)]),
        "rtx_dn_layer": (i, [vp, i, C.POINTER(C.c_int64)]),
        "rtx_dn_get_params": (i, [vp, vp]),
        "rtx_dn_set_params": (i, [vp, vp]),
        "rtx_dn_get_grads": (i, [vp, vp]),
        "rtx_dn_get_adam": (i, [vp, vp, vp]),
        "rtx_dn_set_adam": (i, [vp, vp, vp, i]),
        "rtx_dn_loss_grads": (i, [vp, vp, vp, i, i, i, C.POINTER(C.c_double)]),
        "rtx_dn_train_step": (i, [vp, vp, vp, i, i, i, f, C.POINTER(C.c_double)]),
        "rtx_dn_infer": (i, [vp, vp, vp, i, i, i]),
        "rtx_denoise": (i, [vp, vp, vp, vp, vp, i, vp, i, i]),
        "rtx_scene_set_texture_table": (i, [vp, vp]),
        "rtx_texture_sample": (i, [vp, i, f, i, vp, vp]),
        "rtx_render_pt_resolved": (i, [vp, vp, i, i, i, i, u64, vp, f, f, vp, vp, i]),
        "rtx_image_resolve": (i, [vp, vp, i, i, f, f, vp, vp, i]),
        "rtx_image_tonemap": (i, [vp, vp, vp, i, i, f]),
        "rtx_image_gamma": (i, [vp, vp, vp, i, i, f]),
        "rtx_encode_bmp": (i, [vp, vp, i, i, vp, C.c_size_t, C.POINTER(C.c_size_t)]),
        "rtx_encode_ppm": (i, [vp, vp, i, i, vp, C.c_size_t, C.POINTER(C.c_size_t)]),
        "rtx_obj_import": (i, [C.c_char_p, C.c_char_p, C.POINTER(vp), C.c_char_p, C.c_size_t]),
        "rtx_obj_free": (None, [vp]),
        "rtx_obj_info": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
        "rtx_obj_triangles": (i, [vp, vp, vp, vp, vp]),
        "rtx_obj_mesh": (i, [vp, i, C.POINTER(C.c_char_p), C.POINTER(C.c_uint8), vp, C.POINTER(i)]),
        "rtx_obj_material": (i, [vp, i, C.POINTER(C.c_char_p), vp]),
        "rtx_batch_upload": (i, [vp, i, C.POINTER(SceneDesc)]),
        "rtx_render_batch": (i, [vp, i, C.POINTER(Job), i, vp]),
        "rtx_batch_autotune": (i, [vp, i, C.POINTER(SceneDesc), i, C.POINTER(Job), i, C.POINTER(TuneResult)]),
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


class ObjModel:
    """An OBJ (+ MTL) file imported by rtx_obj_import (no GPU needed): the
    triangle arrays, the meshes (name, smooth flag, Mesh::tris order) and the
    MTL materials.  Names are the file's bytes decoded as UTF-8, with bytes
    that are not UTF-8 kept as surrogate escapes."""

    def __init__(self, obj_path, mtl_path=None):
        L = lib()
        h = C.c_void_p()
        msg = C.create_string_buffer(512)
        r = L.rtx_obj_import(os.fsencode(obj_path), os.fsencode(mtl_path) if mtl_path else None, C.byref(h),
                             msg, 512)
        if r != 0:
            raise RtxError(r, msg.value.decode())
        try:
            nt, nm, nmat = C.c_int(), C.c_int(), C.c_int()
            L.rtx_obj_info(h, C.byref(nt), C.byref(nm), C.byref(nmat))
            n = nt.value
            self.verts = np.zeros((n, 9), np.float32)
            self.norms = np.zeros((n, 9), np.float32)
            self.uvs = np.zeros((n, 6), np.float32)
            self.tri_mesh = np.zeros(n, np.int32)
            L.rtx_obj_triangles(h, _ptr(self.verts), _ptr(self.norms), _ptr(self.uvs), _ptr(self.tri_mesh))
            self.mesh_names, self.mesh_smooth, self.mesh_tris = [], [], []
            for m in range(nm.value):
                name, sm, k = C.c_char_p(), C.c_uint8(), C.c_int()
                L.rtx_obj_mesh(h, m, C.byref(name), C.byref(sm), None, C.byref(k))
                t = np.zeros(k.value, np.int32)
                L.rtx_obj_mesh(h, m, None, None, _ptr(t), C.byref(k))
                self.mesh_names.append(name.value.decode("utf-8", "surrogateescape"))
                self.mesh_smooth.append(sm.value)
                self.mesh_tris.append(t)
            self.material_names, recs = [], []
            for m in range(nmat.value):
                name = C.c_char_p()
                rec = np.zeros(24, np.float32)
                L.rtx_obj_material(h, m, C.byref(name), _ptr(rec))
                self.material_names.append(name.value.decode("utf-8", "surrogateescape"))
                recs.append(rec)
            self.materials = np.stack(recs) if recs else np.zeros((0, 24), np.float32)
        finally:
            L.rtx_obj_free(h)

    def emitter_order(self, mesh_mat, mats):
        """Emitter triangle ids as World::PrepareDirectLightSampling collects
        them (src/world.cpp:24-37): meshes in order, each emissive mesh's
        Mesh::tris in order."""
        out = [self.mesh_tris[m] for m in range(len(self.mesh_names))
               if np.any(np.abs(np.asarray(mats)[mesh_mat[m], 3:6]) > np.float32(1e-7))]
        return np.concatenate(out).astype(np.int32) if out else np.zeros(0, np.int32)


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

    def render_pt_progressive(self, W, H, first_sample, n_samples, spp, max_depth, seed=0, camera=None,
                              out=None):
        """Samples [first_sample, first_sample + n_samples) of an spp-sample
        frame added into `out` (overwritten when first_sample is 0)."""
        cam = self._cam(camera)
        o = np.zeros((H, W, 3), np.float32) if out is None else out
        self._check(self.L.rtx_render_pt_progressive(self.h, _ptr(cam), W, H, first_sample, n_samples, spp,
                                                     max_depth, seed, _ptr(o)))
        return o

    def trace_paths(self, W, H, first_sample, n_samples, max_depth, seed=0, camera=None, out=None):
        cam = self._cam(camera)
        o = np.zeros((n_samples, H * W, 3), np.float32) if out is None else out
        self._check(self.L.rtx_trace_paths(self.h, _ptr(cam), W, H, first_sample, n_samples,
                                           max_depth, seed, _ptr(o)))
        return o

    def aov(self, W, H, near, far, camera=None, out=None):
        """normal, albedo, depth passes (H x W x 3 each); out = three
        preallocated buffers (host arrays or device tensors) or None."""
        cam = self._cam(camera)
        if out is None:
            out = tuple(np.zeros((H, W, 3), np.float32) for _ in range(3))
        n, a, d = out
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

    def bsdf_eval(self, mats, eta, N, V, L):
        """PrincipledBSDF::Eval of n cases on the device: (f [n, 3], pdf [n])."""
        mats = _f32(mats).reshape(-1, 24)
        n = len(mats)
        f = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        args = [_f32(a).reshape(n, -1) for a in (eta, N, V, L)]
        self._check(self.L.rtx_bsdf_eval(self.h, n, _ptr(mats), *[_ptr(a) for a in args], _ptr(f), _ptr(pdf)))
        return f, pdf

    def bsdf_sample(self, mats, eta, N, in_dir, seed, sample):
        """PrincipledBSDF::Sample of n cases on the device (case i draws as
        path (pixel i, sample)): (ok [n], dir [n, 3], color [n, 3], pdf [n])."""
        mats = _f32(mats).reshape(-1, 24)
        n = len(mats)
        ok = np.zeros(n, np.int32)
        od = np.zeros((n, 3), np.float32)
        col = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        args = [_f32(a).reshape(n, -1) for a in (eta, N, in_dir)]
        self._check(self.L.rtx_bsdf_sample(self.h, n, _ptr(mats), *[_ptr(a) for a in args], int(seed),
                                           int(sample), _ptr(ok), _ptr(od), _ptr(col), _ptr(pdf)))
        return ok, od, col, pdf

    def probe_read_bandwidth(self, nbytes, passes):
        """GB/s of a plain streaming read of an nbytes device buffer, `passes`
        times over in one launch (an L2-resident size measures L2)."""
        gbs = C.c_double()
        self._check(self.L.rtx_probe_read_bandwidth(self.h, int(nbytes), int(passes), C.byref(gbs)))
        return gbs.value

    # -- denoiser building blocks ---------------------------------------------
    def gemm_bf16(self, A, B, a_mn=False, b_mn=False, out=None):
        """C = A @ B.T on the tensor cores; A, B are uint16 arrays of BF16 bits
        (or device bfloat16 tensors), M x K and N x K, or K x M / K x N when
        a_mn / b_mn."""
        M, K = (A.shape[1], A.shape[0]) if a_mn else A.shape
        N = B.shape[1] if b_mn else B.shape[0]
        C_ = np.zeros((M, N), np.float32) if out is None else out
        self._check(self.L.rtx_nn_gemm_bf16(self.h, M, N, K, _ptr(A), _ptr(B), _ptr(C_), int(a_mn),
                                            int(b_mn)))
        return C_

    # -- multi-scene batches -------------------------------------------------------
    def batch_upload(self, scene_list, emitters=None):
        """Merge scenes (scenes.Scene) into the context's batch; emitters: per
        scene an explicit emitter id list or None."""
        descs, keep = self._scene_descs(scene_list, emitters)
        self._check(self.L.rtx_batch_upload(self.h, len(scene_list), descs))
        self.batch_scenes = list(scene_list)

    def _scene_descs(self, scene_list, emitters=None):
        keep, descs = [], (SceneDesc * len(scene_list))()
        for k, sc in enumerate(scene_list):
            arrs = [_f32(sc.verts), _f32(sc.norms), np.ascontiguousarray(sc.tri_mesh, np.int32),
                    np.ascontiguousarray(sc.mesh_mat, np.int32), np.ascontiguousarray(sc.mesh_smooth, np.uint8),
                    _f32(sc.mats), _f32(sc.sky), _f32(sc.ground)]
            em = None if emitters is None or emitters[k] is None else np.ascontiguousarray(emitters[k], np.int32)
            keep += arrs + [em]
            v, n, tm, mm, ms, mats, sky, gr = arrs
            descs[k] = SceneDesc(sc.n_tris, v.ctypes.data, n.ctypes.data, tm.ctypes.data, len(mm), mm.ctypes.data,
                                 ms.ctypes.data, len(mats), mats.ctypes.data, sky.ctypes.data, gr.ctypes.data,
                                 None if em is None else em.ctypes.data, -1 if em is None else len(em))
        return descs, keep

    def _jobs(self, jobs):
        arr = (Job * len(jobs))()
        for k, j in enumerate(jobs):
            known = 0 <= j["scene"] < len(getattr(self, "batch_scenes", []))
            cam = _f32(j["camera"] if "camera" in j else
                       (self.batch_scenes[j["scene"]].camera if known else np.zeros(21)))  # rejected by the library
            arr[k] = Job(j["scene"], (C.c_float * 21)(*cam.tolist()), j["W"], j["H"], j["spp"], j.get("seed", 0))
        return arr

    def batch_autotune(self, jobs, max_depth, scene_list=None):
        """Tune leaf size (when scene_list is given: rebuilds), block and wave
        size on the batch frame `jobs`; the best stays set.  Returns a dict."""
        descs, keep = (None, None) if scene_list is None else self._scene_descs(scene_list)
        res = TuneResult()
        self._check(self.L.rtx_batch_autotune(self.h, 0 if scene_list is None else len(scene_list), descs,
                                              len(jobs), self._jobs(jobs), max_depth, C.byref(res)))
        if scene_list is not None:
            self.batch_scenes = list(scene_list)
        return {k: getattr(res, k) for k, _ in TuneResult._fields_}

    def render_batch(self, jobs, max_depth, out=None):
        """jobs: dicts with scene (index), W, H, spp, seed and optionally camera
        (default: the scene's).  Returns the list of H x W x 3 images (views of
        one buffer), or fills `out` (a flat device tensor or array)."""
        arr = self._jobs(jobs)
        total = sum(j["W"] * j["H"] for j in jobs)
        buf = np.zeros(total * 3, np.float32) if out is None else out
        self._check(self.L.rtx_render_batch(self.h, len(jobs), arr, max_depth, _ptr(buf)))
        if out is not None:
            return out
        imgs, o = [], 0
        for j in jobs:
            n = j["W"] * j["H"] * 3
            imgs.append(buf[o:o + n].reshape(j["H"], j["W"], 3))
            o += n
        return imgs

    # -- display resolve and image files -------------------------------------------
    BYTES_BMP, BYTES_RGB = 0, 1

    @staticmethod
    def _byte_buf(W, H, fmt):
        n = ((3 * W + 3) & ~3) * H if fmt == 0 else 3 * W * H
        return np.zeros(n, np.uint8)

    def render_pt_resolved(self, W, H, spp, max_depth, seed=0, limit=1.5, gamma=2.2, fmt=1,
                           want_display=True, want_bytes=True, camera=None):
        cam = self._cam(camera)
        o = np.zeros((H, W, 3), np.float32)
        disp = np.zeros((H, W, 3), np.float32) if want_display else None
        byt = self._byte_buf(W, H, fmt) if want_bytes else None
        self._check(self.L.rtx_render_pt_resolved(self.h, _ptr(cam), W, H, spp, max_depth, seed, _ptr(o),
                                                  limit, gamma, _ptr(disp), _ptr(byt), fmt))
        return o, disp, byt

    def resolve(self, img, limit=1.5, gamma=2.2, fmt=1, want_display=True, want_bytes=True):
        img = img if hasattr(img, "data_ptr") else _f32(img)
        H, W = int(img.shape[0]), int(img.shape[1])
        disp = np.zeros((H, W, 3), np.float32) if want_display else None
        byt = self._byte_buf(W, H, fmt) if want_bytes else None
        self._check(self.L.rtx_image_resolve(self.h, _ptr(img), W, H, limit, gamma, _ptr(disp), _ptr(byt), fmt))
        return disp, byt

    def tonemap(self, img, limit=1.5, out=None):
        img, out, W, H = self._img_io(img, out)
        self._check(self.L.rtx_image_tonemap(self.h, _ptr(img), _ptr(out), W, H, limit))
        return out

    def gamma(self, img, gamma=2.2, out=None):
        img, out, W, H = self._img_io(img, out)
        self._check(self.L.rtx_image_gamma(self.h, _ptr(img), _ptr(out), W, H, gamma))
        return out

    def _encode(self, fn, img):
        img = _f32(img)
        H, W = img.shape[:2]
        n = C.c_size_t()
        self._check(fn(self.h, _ptr(img), W, H, None, 0, C.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        self._check(fn(self.h, _ptr(img), W, H, _ptr(buf), n.value, C.byref(n)))
        return buf.tobytes()

    def encode_bmp(self, img):
        """BMPExporter output (bytes) of an H x W x 3 image."""
        return self._encode(self.L.rtx_encode_bmp, img)

    def encode_ppm(self, img):
        """PPMExporter output (bytes) of an H x W x 3 image."""
        return self._encode(self.L.rtx_encode_ppm, img)

    # -- procedural textures ------------------------------------------------------
    def set_texture_table(self, perm):
        perm = np.ascontiguousarray(perm, np.uint8)
        assert perm.size == 256
        self._check(self.L.rtx_scene_set_texture_table(self.h, _ptr(perm)))

    def texture_sample(self, kind, param, uv):
        uv = _f32(uv).reshape(-1, 2)
        out = np.zeros(len(uv), np.float32)
        self._check(self.L.rtx_texture_sample(self.h, int(kind), float(param), len(uv), _ptr(uv), _ptr(out)))
        return out

    # -- denoiser operators -------------------------------------------------------
    def conv3x3_fwd(self, x1, w, Cout, x2=None, up1=False, bias=None, relu=False, out=None):
        """One convolution of the denoiser: x1 [N][h][w][C1] (half resolution
        when up1), x2 [N][H][W][C2], w [Cout][9][C1 + C2], all BF16 bits
        (uint16) or device bfloat16 tensors; returns FP32 [N][H][W][Cout]."""
        N, H, W, C1 = x1.shape
        if up1:
            H, W = 2 * H, 2 * W
        C2 = 0 if x2 is None else x2.shape[3]
        if out is None:
            out = np.zeros((N, H, W, Cout), np.float32)
        b = None if bias is None else (bias if hasattr(bias, "data_ptr") else _f32(bias))
        self._check(self.L.rtx_nn_conv3x3_fwd(self.h, N, H, W, _ptr(x1), C1, int(up1), _ptr(x2), C2, _ptr(w),
                                              _ptr(b), Cout, int(relu), _ptr(out)))
        return out

    def conv3x3_dgrad(self, dout, wt, x1, x2=None, up1=False, mask_relu=False, out=None):
        """din [N][H][W][C1 + C2] (BF16 bits) of a convolution; wt [Cin][9][Cout]."""
        N, H, W, Cout = dout.shape
        C1 = x1.shape[3]
        C2 = 0 if x2 is None else x2.shape[3]
        if out is None:
            out = np.zeros((N, H, W, C1 + C2), np.uint16)
        self._check(self.L.rtx_nn_conv3x3_dgrad(self.h, N, H, W, _ptr(dout), Cout, _ptr(wt), _ptr(x1), C1,
                                                int(up1), _ptr(x2), C2, int(mask_relu), _ptr(out)))
        return out

    def conv3x3_wgrad(self, dout, x1, x2=None, up1=False, out=None):
        """dw [Cout][9][C1 + C2] (FP32) of a convolution."""
        N, H, W, Cout = dout.shape
        C1 = x1.shape[3]
        C2 = 0 if x2 is None else x2.shape[3]
        if out is None:
            out = np.zeros((Cout, 9, C1 + C2), np.float32)
        self._check(self.L.rtx_nn_conv3x3_wgrad(self.h, N, H, W, _ptr(dout), Cout, _ptr(x1), C1, int(up1),
                                                _ptr(x2), C2, _ptr(out)))
        return out

    # -- denoiser ---------------------------------------------------------------
    def dn_init(self, seed=0):
        self._check(self.L.rtx_dn_init(self.h, seed))

    def dn_info(self):
        n, r, nl, st = C.c_int64(), C.c_int64(), C.c_int(), C.c_int()
        self._check(self.L.rtx_dn_info(self.h, C.byref(n), C.byref(r), C.byref(nl), C.byref(st)))
        return {"n_params": n.value, "n_real": r.value, "n_layers": nl.value, "step": st.value}

    DN_LAYER_KEYS = ("cout_pad", "cout", "cin_pad", "cin", "c1_pad", "up1", "relu", "level", "w_off",
                     "b_off", "src1")

    def dn_layers(self):
        out = []
        for i in range(self.dn_info()["n_layers"]):
            a = (C.c_int64 * 11)()
            self._check(self.L.rtx_dn_layer(self.h, i, a))
            out.append(dict(zip(self.DN_LAYER_KEYS, list(a))))
        return out

    def dn_get_params(self):
        p = np.zeros(self.dn_info()["n_params"], np.float32)
        self._check(self.L.rtx_dn_get_params(self.h, _ptr(p)))
        return p

    def dn_set_params(self, p):
        p = _f32(p)
        assert p.size == self.dn_info()["n_params"]
        self._check(self.L.rtx_dn_set_params(self.h, _ptr(p)))

    def dn_get_grads(self):
        g = np.zeros(self.dn_info()["n_params"], np.float32)
        self._check(self.L.rtx_dn_get_grads(self.h, _ptr(g)))
        return g

    def dn_get_adam(self):
        n = self.dn_info()["n_params"]
        m, v = np.zeros(n, np.float32), np.zeros(n, np.float32)
        self._check(self.L.rtx_dn_get_adam(self.h, _ptr(m), _ptr(v)))
        return m, v

    def dn_set_adam(self, m, v, step):
        m, v = _f32(m), _f32(v)
        self._check(self.L.rtx_dn_set_adam(self.h, _ptr(m), _ptr(v), int(step)))

    @staticmethod
    def _batch(x):
        if x.ndim == 3:
            x = x[None]
        return x if hasattr(x, "data_ptr") else _f32(x)

    def dn_loss_grads(self, inp, target):
        """Loss of a batch (inp [N][H][W][11], target [N][H][W][3]); the
        gradients are then read with dn_get_grads."""
        inp, target = self._batch(inp), self._batch(target)
        N, H, W = inp.shape[:3]
        l = C.c_double()
        self._check(self.L.rtx_dn_loss_grads(self.h, _ptr(inp), _ptr(target), N, H, W, C.byref(l)))
        return l.value

    def dn_train_step(self, inp, target, lr=3e-4):
        inp, target = self._batch(inp), self._batch(target)
        N, H, W = inp.shape[:3]
        l = C.c_double()
        self._check(self.L.rtx_dn_train_step(self.h, _ptr(inp), _ptr(target), N, H, W, float(lr),
                                             C.byref(l)))
        return l.value

    def dn_infer(self, inp, out=None):
        inp = self._batch(inp)
        N, H, W = inp.shape[:3]
        if out is None:
            out = np.zeros((N, H, W, 3), np.float32)
        self._check(self.L.rtx_dn_infer(self.h, _ptr(inp), _ptr(out), N, H, W))
        return out

    def denoise(self, radiance, albedo, normal, depth, spp, out=None):
        """Denoise a frame from its passes (each H x W x 3 FP32), the radiance
        rendered at `spp` samples per pixel."""
        rad, alb, nrm, dep = (x if hasattr(x, "data_ptr") else _f32(x) for x in (radiance, albedo, normal, depth))
        H, W = rad.shape[:2]
        if out is None:
            out = np.zeros((H, W, 3), np.float32)
        self._check(self.L.rtx_denoise(self.h, _ptr(rad), _ptr(alb), _ptr(nrm), _ptr(dep), int(spp), _ptr(out),
                                       W, H))
        return out

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
