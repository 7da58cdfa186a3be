"""ctypes binding of the CPU checkers (TEST INFRASTRUCTURE ONLY).

``load("oracle")`` binds oracle/_build/liboracle.so (the restatement, built on
every machine by ``make -C oracle``).  ``load("ref")`` / ``load("ref_orig")``
bind oracle/_ref/libref*.so, the reference's own sources linked with
oracle/ref_harness.cpp; those exist only where the RenderToy sources are
present (``make -C oracle ref``).  All expose the same API (rt_oracle.h).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATHS = {
    "oracle": os.path.join(HERE, "_build", "liboracle.so"),
    "ref": os.path.join(HERE, "_ref", "libref.so"),
    "ref_orig": os.path.join(HERE, "_ref", "libref_orig.so"),
}

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build(ref: bool = False) -> None:
    subprocess.check_call(["make", "-s", "-C", HERE] + (["ref"] if ref else []))


def _opt(a, dt):
    return None if a is None else np.ascontiguousarray(a, dt)


class Checker:
    """One loaded checker library (prefix 'orc' or 'ref')."""

    def __init__(self, kind: str = "oracle"):
        path = PATHS[kind]
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built (make -C oracle{' ref' if kind != 'oracle' else ''})")
        self.kind = kind
        self.lib = C.CDLL(path)
        p = "orc_" if kind == "oracle" else "ref_"
        self.p = p
        L = self.lib
        self._fn = {}

        def fn(name, res, args):
            f = getattr(L, p + name)
            f.restype = res
            f.argtypes = args
            self._fn[name] = f

        vp = C.c_void_p
        fn("scene_create", vp, [C.c_int, _f32p, vp, _i32p, C.c_int, _i32p, _u8p, C.c_int,
                                _f32p, _f32p, _f32p])
        fn("scene_destroy", None, [vp])
        fn("scene_emitters", C.c_int, [vp, _i32p, C.c_int])
        fn("intersect", None, [vp, C.c_int, _f32p, vp, _i32p, _f32p, C.c_int])
        fn("primary", None, [vp, _f32p, C.c_int, C.c_int, _i32p, _f32p, C.c_int])
        fn("render_aov", None, [vp, _f32p, C.c_int, C.c_int, C.c_float, C.c_float, vp, vp, vp, C.c_int])
        fn("trace_paths", None, [vp, _f32p, C.c_int, C.c_int, vp, C.c_int, C.c_int, C.c_int,
                                 C.c_int, C.c_uint64, _f32p, C.c_int])
        fn("bsdf_eval", None, [_f32p, C.c_float, _f32p, _f32p, _f32p, _f32p, _f32p])
        fn("bsdf_sample", C.c_int, [_f32p, C.c_float, _f32p, _f32p, C.c_uint64, C.c_uint32,
                                    C.c_uint32, _f32p, _f32p, _f32p])
        fn("convolve", None, [_f32p, _f32p, C.c_int, C.c_int, _f32p, C.c_int, C.c_int,
                              C.c_int, C.c_int, C.c_int])
        fn("gaussian_blur", None, [_f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_float])
        fn("gaussian_weights", None, [C.c_int, C.c_float, _f32p])
        fn("edge_detect", None, [_f32p, _f32p, C.c_int, C.c_int])
        fn("bloom", None, [_f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float])
        fn("rng_floats", None, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_int, _f32p])
        fn("texture_sample", None, [C.c_int, C.c_float, vp, C.c_int, _f32p, _f32p])
        fn("tonemap_gamma", None, [_f32p, C.c_int, C.c_int, C.c_float, C.c_float, _f32p])
        fn("encode", C.c_long, [C.c_int, _f32p, C.c_int, C.c_int, _u8p, C.c_long])
        if kind == "oracle":
            fn("scene_set_texture_table", None, [vp, _u8p])
        else:
            fn("perlin_table", None, [_u8p])
            fn("obj_import", vp, [C.c_char_p, C.c_char_p])
            fn("obj_counts", None, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)])
            fn("obj_arrays", None, [vp, _f32p, _f32p, _f32p, _i32p, _u8p, _i32p, _i32p, _f32p])
            fn("obj_mesh_name", C.c_char_p, [vp, C.c_int])
            fn("obj_mat_name", C.c_char_p, [vp, C.c_int])
            fn("obj_free", None, [vp])
        if kind == "oracle":
            fn("render_pt", None, [vp, _f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64,
                                   _f32p, C.c_int])
        else:
            fn("render_pt", C.c_double, [vp, _f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp])

    # -- scene -------------------------------------------------------------
    def scene(self, sc):
        return CheckerScene(self, sc)

    # -- procedural textures ------------------------------------------------
    def texture_sample(self, kind, param, uv, perm=None):
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        out = np.zeros(len(uv), np.float32)
        pp = None if perm is None else np.ascontiguousarray(perm, np.uint8)
        self._fn["texture_sample"](int(kind), float(param), None if pp is None else pp.ctypes.data,
                                   len(uv), uv, out)
        return out

    def tonemap_gamma(self, img, limit, gamma):
        img = np.ascontiguousarray(img, np.float32)
        out = np.zeros_like(img)
        self._fn["tonemap_gamma"](img, img.shape[1], img.shape[0], float(limit), float(gamma), out)
        return out

    def encode(self, img, bmp):
        img = np.ascontiguousarray(img, np.float32)
        H, W = img.shape[:2]
        n = self._fn["encode"](int(bmp), img, W, H, np.zeros(1, np.uint8), 0)
        assert n >= 0, "not encodable by this checker"
        buf = np.zeros(n, np.uint8)
        self._fn["encode"](int(bmp), img, W, H, buf, n)
        return buf.tobytes()

    def obj_import(self, obj_path, mtl_path=None):
        """RenderToy's OBJModelImporter (+ MTLImporter) read back as arrays."""
        h = self._fn["obj_import"](os.fsencode(obj_path), os.fsencode(mtl_path) if mtl_path else None)
        try:
            nt, nm, nmat = C.c_int(), C.c_int(), C.c_int()
            self._fn["obj_counts"](h, C.byref(nt), C.byref(nm), C.byref(nmat))
            n = nt.value
            out = dict(verts=np.zeros((n, 9), np.float32), norms=np.zeros((n, 9), np.float32),
                       uvs=np.zeros((n, 6), np.float32), tri_mesh=np.zeros(n, np.int32),
                       mesh_smooth=np.zeros(nm.value, np.uint8), mesh_counts=np.zeros(nm.value, np.int32),
                       mesh_tris=np.zeros(n + 1, np.int32), materials=np.zeros((max(nmat.value, 1), 24), np.float32))
            self._fn["obj_arrays"](h, out["verts"], out["norms"], out["uvs"], out["tri_mesh"], out["mesh_smooth"],
                                   out["mesh_counts"], out["mesh_tris"], out["materials"])
            out["mesh_tris"] = out["mesh_tris"][:int(out["mesh_counts"].sum())]
            out["materials"] = out["materials"][:nmat.value]
            out["mesh_names"] = [self._fn["obj_mesh_name"](h, i).decode() for i in range(nm.value)]
            out["material_names"] = [self._fn["obj_mat_name"](h, i).decode() for i in range(nmat.value)]
            return out
        finally:
            self._fn["obj_free"](h)

    def perlin_table(self):
        out = np.zeros(256, np.uint8)
        self._fn["perlin_table"](out)
        return out

    # -- BSDF --------------------------------------------------------------
    def bsdf_eval(self, mat, eta, N, V, L):
        f = np.zeros(3, np.float32)
        pdf = np.zeros(1, np.float32)
        self._fn["bsdf_eval"](np.ascontiguousarray(mat, np.float32), float(eta),
                              np.ascontiguousarray(N, np.float32), np.ascontiguousarray(V, np.float32),
                              np.ascontiguousarray(L, np.float32), f, pdf)
        return f, pdf[0]

    def bsdf_sample(self, mat, eta, N, in_dir, seed, pixel, sample):
        od = np.zeros(3, np.float32)
        col = np.zeros(3, np.float32)
        pdf = np.zeros(1, np.float32)
        ok = self._fn["bsdf_sample"](np.ascontiguousarray(mat, np.float32), float(eta),
                                     np.ascontiguousarray(N, np.float32),
                                     np.ascontiguousarray(in_dir, np.float32), seed, pixel, sample,
                                     od, col, pdf)
        return ok, od, col, pdf[0]

    # -- compositor --------------------------------------------------------
    def convolve(self, img, k, normalize=False, length=False, absval=False):
        H, W = img.shape[:2]
        k = np.ascontiguousarray(k, np.float32)
        out = np.zeros_like(img, dtype=np.float32)
        self._fn["convolve"](np.ascontiguousarray(img, np.float32), out, W, H, k, k.shape[0],
                             k.shape[1], int(normalize), int(length), int(absval))
        return out

    def gaussian_blur(self, img, size, sigma):
        H, W = img.shape[:2]
        out = np.zeros_like(img, dtype=np.float32)
        self._fn["gaussian_blur"](np.ascontiguousarray(img, np.float32), out, W, H, size, sigma)
        return out

    def gaussian_weights(self, size, sigma):
        out = np.zeros(size, np.float32)
        self._fn["gaussian_weights"](size, sigma, out)
        return out

    def edge_detect(self, img):
        H, W = img.shape[:2]
        out = np.zeros_like(img, dtype=np.float32)
        self._fn["edge_detect"](np.ascontiguousarray(img, np.float32), out, W, H)
        return out

    def bloom(self, img, size, sigma, threshold):
        H, W = img.shape[:2]
        out = np.zeros_like(img, dtype=np.float32)
        self._fn["bloom"](np.ascontiguousarray(img, np.float32), out, W, H, size, sigma, threshold)
        return out

    def rng_floats(self, seed, pixel, sample, n):
        out = np.zeros(n, np.float32)
        self._fn["rng_floats"](seed, pixel, sample, n, out)
        return out


class CheckerScene:
    def __init__(self, chk: Checker, sc):
        self.chk = chk
        self.sc = sc
        norms = np.ascontiguousarray(sc.norms, np.float32)
        self._keep = norms
        self.h = chk._fn["scene_create"](
            sc.n_tris, np.ascontiguousarray(sc.verts, np.float32), norms.ctypes.data,
            np.ascontiguousarray(sc.tri_mesh, np.int32), len(sc.mesh_mat),
            np.ascontiguousarray(sc.mesh_mat, np.int32), np.ascontiguousarray(sc.mesh_smooth, np.uint8),
            len(sc.mats), np.ascontiguousarray(sc.mats, np.float32),
            np.ascontiguousarray(sc.sky, np.float32), np.ascontiguousarray(sc.ground, np.float32))

    def set_texture_table(self, perm):
        self.chk._fn["scene_set_texture_table"](self.h, np.ascontiguousarray(perm, np.uint8))

    def close(self):
        if self.h:
            self.chk._fn["scene_destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def emitters(self):
        out = np.zeros(max(self.sc.n_tris, 1), np.int32)
        n = self.chk._fn["scene_emitters"](self.h, out, len(out))
        return out[:n].copy()

    def intersect(self, rays, exclude=None, threads=0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = len(rays)
        ex = _opt(exclude, np.int32)
        tri = np.zeros(n, np.int32)
        tuv = np.zeros((n, 3), np.float32)
        self.chk._fn["intersect"](self.h, n, rays, None if ex is None else ex.ctypes.data, tri, tuv,
                                  threads)
        return tri, tuv

    def primary(self, W, H, cam=None, threads=0):
        cam = self.sc.camera if cam is None else cam
        tri = np.zeros(W * H, np.int32)
        tuv = np.zeros((W * H, 3), np.float32)
        self.chk._fn["primary"](self.h, np.ascontiguousarray(cam, np.float32), W, H, tri, tuv, threads)
        return tri.reshape(H, W), tuv.reshape(H, W, 3)

    def aov(self, W, H, near, far, cam=None, threads=0):
        cam = self.sc.camera if cam is None else cam
        n = np.zeros((H, W, 3), np.float32)
        a = np.zeros((H, W, 3), np.float32)
        d = np.zeros((H, W, 3), np.float32)
        self.chk._fn["render_aov"](self.h, np.ascontiguousarray(cam, np.float32), W, H, near, far,
                                   n.ctypes.data, a.ctypes.data, d.ctypes.data, threads)
        return n, a, d

    def trace_paths(self, W, H, first_sample, n_samples, max_depth, seed, pixels=None, cam=None,
                    threads=0):
        cam = self.sc.camera if cam is None else cam
        px = _opt(pixels, np.int32)
        npix = W * H if px is None else len(px)
        out = np.zeros((n_samples, npix, 3), np.float32)
        self.chk._fn["trace_paths"](self.h, np.ascontiguousarray(cam, np.float32), W, H,
                                    None if px is None else px.ctypes.data, npix, first_sample,
                                    n_samples, max_depth, seed, out, threads)
        return out

    def render_pt(self, W, H, spp, max_depth, seed, cam=None, threads=0):
        cam = self.sc.camera if cam is None else cam
        out = np.zeros((H, W, 3), np.float32)
        if self.chk.kind != "oracle":
            raise ValueError("the reference renders with Render(); use render_native")
        self.chk._fn["render_pt"](self.h, np.ascontiguousarray(cam, np.float32), W, H, spp,
                                  max_depth, seed, out, threads)
        return out

    def render_native(self, W, H, spp, max_depth, cam=None, threads=0):
        """The reference's own PathTracingRenderer::Render (reference builds
        only): (image, seconds inside Render)."""
        cam = self.sc.camera if cam is None else cam
        out = np.zeros((H, W, 3), np.float32)
        sec = self.chk._fn["render_pt"](self.h, np.ascontiguousarray(cam, np.float32), W, H, spp,
                                        max_depth, threads, out.ctypes.data)
        return out, sec


def load(kind: str = "oracle") -> Checker:
    return Checker(kind)
