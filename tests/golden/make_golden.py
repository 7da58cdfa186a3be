"""Generate the golden vectors in tests/golden/ from RenderToy's OWN code.

Run where the RenderToy sources are present (they are read, never copied):

    python tests/golden/make_golden.py [--ref /path/to/RenderToy]

It builds oracle/_ref/libref.so (reference sources with the recursion cap as a
parameter, RNG wrapped) and oracle/_ref/libref_orig.so (unmodified sources) via
``make -C oracle ref``, runs both on seeded synthetic inputs, checks that the
patched build at the reference cap equals the unmodified one and that the
restatement (oracle/_build/liboracle.so) equals the reference bit for bit, and
writes the reference's outputs as .npz fixtures.  The tests compare the oracle
with these fixtures on every machine, and the CUDA path with the oracle.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import bind  # noqa: E402
from rendertoy_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SEED = 7


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def check_equal(name, a, b, mask=None):
    a, b = bits(a), bits(b)
    if mask is not None:
        a, b = a[mask], b[mask]
    ok = np.array_equal(a, b)
    print(f"  {name}: {'bit-exact' if ok else 'MISMATCH'}")
    if not ok:
        raise SystemExit(f"oracle differs from the reference on {name}")


def scene_case(ref, refo, orc, sc, W, H, tag):
    rs, ro, os_ = ref.scene(sc), refo.scene(sc), orc.scene(sc)
    near, far = float(sc.camera[19]), float(sc.camera[20])
    out = dict(verts=sc.verts, norms=sc.norms, tri_mesh=sc.tri_mesh, mesh_mat=sc.mesh_mat,
               mesh_smooth=sc.mesh_smooth, mats=sc.mats, sky=sc.sky, ground=sc.ground,
               camera=sc.camera, W=W, H=H, seed=SEED)
    em = rs.emitters()
    assert np.array_equal(em, sc.emitters()), "emitter order"
    assert np.array_equal(em, os_.emitters())
    out["emitters"] = em
    tri, tuv = rs.primary(W, H)
    t2, u2 = os_.primary(W, H)
    assert np.array_equal(tri, t2)
    check_equal(f"{tag} primary t/u/v", tuv, u2)
    out["primary_tri"], out["primary_tuv"] = tri, tuv
    n, a, d = rs.aov(W, H, near, far)
    n2, a2, d2 = os_.aov(W, H, near, far)
    check_equal(f"{tag} normal", n, n2)
    check_equal(f"{tag} albedo", a, a2)
    check_equal(f"{tag} depth", d, d2)
    out["aov_normal"], out["aov_albedo"], out["aov_depth"] = n, a, d
    for depth, spp in ((5, 2), (8, 2)):
        p = rs.trace_paths(W, H, 0, spp, depth, SEED)
        if depth == 5:
            p0 = ro.trace_paths(W, H, 0, spp, depth, SEED)
            check_equal(f"{tag} patched cap == unmodified (depth 5)", p, p0)
        p2 = os_.trace_paths(W, H, 0, spp, depth, SEED)
        check_equal(f"{tag} paths depth {depth}", p, p2)
        out[f"paths_d{depth}"] = p
    np.savez_compressed(os.path.join(OUT, f"scene_{tag}.npz"), **out)


def intersect_case(ref, orc, sc, n=4096):
    rng = np.random.RandomState(11)
    o = rng.uniform(5, 550, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # a quarter of the rays start on a triangle (barycentric point) and
    # exclude it, as bounce and shadow rays do
    k = n // 4
    tid = rng.randint(0, sc.n_tris, k)
    uv = rng.uniform(0, 1, (k, 2))
    swap = uv.sum(1) > 1
    uv[swap] = 1 - uv[swap]
    v = sc.verts[tid].reshape(k, 3, 3).astype(np.float64)
    o[:k] = (v[:, 0] + uv[:, :1] * (v[:, 1] - v[:, 0]) + uv[:, 1:] * (v[:, 2] - v[:, 0])).astype(np.float32)
    ex = np.full(n, -1, np.int32)
    ex[:k] = tid
    rays = np.concatenate([o, d], 1).astype(np.float32)
    rs, os_ = ref.scene(sc), orc.scene(sc)
    t1, u1 = rs.intersect(rays, ex)
    t2, u2 = os_.intersect(rays, ex)
    assert np.array_equal(t1, t2)
    check_equal("intersect t/u/v", u1, u2)
    np.savez_compressed(os.path.join(OUT, "intersect_mixed.npz"), rays=rays, exclude=ex, tri=t1, tuv=u1)


def bsdf_case(ref, orc, n=3000):
    rng = np.random.RandomState(5)
    mats = np.stack([scenes.material(
        base_color=tuple(rng.uniform(0, 1, 3)), roughness=rng.uniform(0.001, 1.0),
        metallic=rng.choice([0.0, 1.0, rng.uniform()]), subsurface=rng.uniform(),
        specular_tint=rng.uniform(), sheen=rng.uniform(), sheen_tint=rng.uniform(),
        clearcoat=rng.choice([0.0, rng.uniform()]), clearcoat_roughness=rng.uniform(0.001, 1.0),
        spec_trans=rng.choice([0.0, 1.0, rng.uniform()]), ior=rng.uniform(1.05, 2.0))
        for _ in range(n)])
    eta = np.where(rng.uniform(size=n) < 0.5, 1.0 / mats[:, 16], mats[:, 16]).astype(np.float32)

    def unit(m):
        v = rng.normal(size=(m, 3))
        return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)

    N, V, L = unit(n), unit(n), unit(n)
    V = np.where((np.sum(V * N, 1) < 0)[:, None], -V, V).astype(np.float32)
    ef, ep = np.zeros((n, 3), np.float32), np.zeros(n, np.float32)
    ok, od, col, sp = (np.zeros(n, np.int32), np.zeros((n, 3), np.float32),
                       np.zeros((n, 3), np.float32), np.zeros(n, np.float32))
    for i in range(n):
        f, p = ref.bsdf_eval(mats[i], eta[i], N[i], V[i], L[i])
        f2, p2 = orc.bsdf_eval(mats[i], eta[i], N[i], V[i], L[i])
        assert np.array_equal(bits(f), bits(f2)) and bits(p) == bits(p2), ("eval", i)
        ef[i], ep[i] = f, p
        r = ref.bsdf_sample(mats[i], eta[i], N[i], V[i], SEED, i, 3)
        r2 = orc.bsdf_sample(mats[i], eta[i], N[i], V[i], SEED, i, 3)
        assert r[0] == r2[0] and all(np.array_equal(bits(x), bits(y)) for x, y in zip(r[1:], r2[1:])), ("sample", i)
        ok[i], od[i], col[i], sp[i] = r
    print(f"  bsdf eval/sample ({n} cases): bit-exact; sample ok fraction {ok.mean():.3f}")
    np.savez_compressed(os.path.join(OUT, "bsdf.npz"), mats=mats, eta=eta, N=N, V=V, L=L,
                        eval_f=ef, eval_pdf=ep, sample_ok=ok, sample_dir=od, sample_color=col,
                        sample_pdf=sp, seed=SEED)


def valid_rows(H, radius):
    """Rows whose taps stay inside the buffer in the reference (its reflect
    index can read one row past the end: include/RenderToy/compositor.h:25-39)."""
    m = np.zeros(H, bool)
    m[: max(H - 1 - radius, 0)] = True
    return m


def compositor_case(ref, orc):
    rng = np.random.RandomState(3)
    out = {}
    for tag, (W, H) in (("a", (37, 29)), ("b", (64, 64))):
        img = (rng.exponential(0.6, (H, W, 3)) * (rng.uniform(size=(H, W, 1)) < 0.9)).astype(np.float32)
        out[f"img_{tag}"] = img
        cases = {
            "blur7": (lambda c: c.gaussian_blur(img, 7, 1.5), 3),
            "blur49": (lambda c: c.gaussian_blur(img, 49, 8.0), 24),
            "edge": (lambda c: c.edge_detect(img), 1),
            "bloom": (lambda c: c.bloom(img, 9, 2.0, 0.8), 4),
        }
        k5 = rng.normal(size=(5, 5)).astype(np.float32)
        out[f"k5_{tag}"] = k5
        for flags in ((0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0), (0, 1, 1)):
            cases[f"conv5_{''.join(map(str, flags))}"] = (
                lambda c, f=flags: c.convolve(img, k5, normalize=f[0], length=f[1], absval=f[2]), 2)
        for name, (fn, radius) in cases.items():
            a, b = fn(ref), fn(orc)
            rows = valid_rows(H, radius)
            check_equal(f"compositor {tag}/{name}", a, b, mask=rows)
            out[f"{name}_{tag}"] = np.where(rows[:, None, None], a, np.float32(0))
            out[f"rows_{name}_{tag}"] = rows
    for size, sigma in ((3, 0.8), (7, 1.5), (49, 8.0), (9, 2.0)):
        w = ref.gaussian_weights(size, sigma)
        check_equal(f"gaussian weights {size}/{sigma}", w, orc.gaussian_weights(size, sigma))
        out[f"gw_{size}"] = w
    np.savez_compressed(os.path.join(OUT, "compositor.npz"), **out)


def rng_case(ref, orc):
    out = {}
    for (seed, pixel, sample) in ((0, 0, 0), (7, 12345, 3), (2**40 + 5, 2**31, 1023)):
        a = ref.rng_floats(seed, pixel, sample, 64)
        check_equal(f"rng {seed}/{pixel}/{sample}", a, orc.rng_floats(seed, pixel, sample, 64))
        out[f"rng_{seed}_{pixel}_{sample}"] = a
    np.savez_compressed(os.path.join(OUT, "rng.npz"), **out)


def write_scene_file(sc, path):
    """Scene file read by tests/compat/demo_cornell.cpp."""
    with open(path, "wb") as f:
        np.array([sc.n_tris, len(sc.mesh_mat), len(sc.mats)], np.int32).tofile(f)
        np.ascontiguousarray(sc.verts, np.float32).tofile(f)
        np.ascontiguousarray(sc.norms, np.float32).tofile(f)
        np.ascontiguousarray(sc.tri_mesh, np.int32).tofile(f)
        np.ascontiguousarray(sc.mesh_mat, np.int32).tofile(f)
        np.ascontiguousarray(sc.mesh_smooth, np.uint8).tofile(f)
        np.ascontiguousarray(sc.mats, np.float32).tofile(f)
        np.ascontiguousarray(sc.camera, np.float32).tofile(f)


def read_demo_output(path):
    with open(path, "rb") as f:
        W, H, n = np.fromfile(f, np.int32, 3)
        return np.fromfile(f, np.float32).reshape(n, H, W, 3)


DEMO_W, DEMO_H, DEMO_SPP = 40, 32, 256


def demo_case(ref_root):
    """tests/compat/demo_cornell.cpp built against RenderToy's own headers and
    sources (serially: no OpenMP), run on the mixed-material scene."""
    rdir = os.path.join(ROOT, "oracle", "_ref")
    os.makedirs(rdir, exist_ok=True)
    exe = os.path.join(rdir, "demo_cornell_ref")
    srcs = [os.path.join(ref_root, "src", f + ".cpp") for f in
            ("bvh", "object", "material", "rtmath", "surfacepoint", "world", "ray", "compositor",
             "exception", "procedural", "importer", "exporter", "renderer")]
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-include", "functional",
                           "-include", "vector", "-include", "cstdint", "-include", "optional",
                           "-include", "algorithm", "-I" + os.path.join(ref_root, "include"),
                           os.path.join(ROOT, "tests", "compat", "demo_cornell.cpp"), *srcs, "-o", exe])
    sc = scenes.cornell_mixed()
    scene_file = os.path.join(rdir, "demo_scene.bin")
    write_scene_file(sc, scene_file)
    out_file = os.path.join(rdir, "demo_out_ref.bin")
    subprocess.check_call([exe, scene_file, out_file, str(DEMO_W), str(DEMO_H), str(DEMO_SPP)])
    out = read_demo_output(out_file)
    np.savez_compressed(os.path.join(OUT, "demo_cornell.npz"), buffers=out, W=DEMO_W, H=DEMO_H,
                        spp=DEMO_SPP)
    print(f"  demo_cornell (reference build): {out.shape[0]} buffers")


TEXTURES = [(1, 4.0), (1, 7.0), (2, 2.5), (2, 0.75), (3, 10.0), (3, 3.0)]


def texture_case(ref, orc):
    """ProceduralTexture::{CheckerBoard, Wave, PerlinNoise}::Sample
    (src/procedural.cpp:8-46) at seeded points, with the permutation a
    default-constructed PerlinNoise uses."""
    rng = np.random.RandomState(SEED)
    uv = np.concatenate([rng.uniform(-3, 3, (4000, 2)), rng.uniform(-300, 300, (64, 2)),
                         np.array([[0, 0], [-0.0, 0.5], [1, 1], [-1, -1], [0.25, -0.25], [2.5, 3.5]])])
    uv = uv.astype(np.float32)
    perm = ref.perlin_table()
    out = {"uv": uv, "perm": perm, "kinds": np.array([k for k, _ in TEXTURES], np.int32),
           "params": np.array([p for _, p in TEXTURES], np.float32)}
    for i, (k, prm) in enumerate(TEXTURES):
        a = ref.texture_sample(k, prm, uv)
        check_equal(f"texture kind {k} param {prm}", orc.texture_sample(k, prm, uv, perm=perm), a)
        out[f"out{i}"] = a
    np.savez_compressed(os.path.join(OUT, "textures.npz"), **out)


def resolve_case(ref, orc):
    """Image::Tonemap / GammaCorrection (compositor.h:220-226,
    compositor.cpp:94-100) and BMPExporter / PPMExporter (exporter.cpp) on a
    seeded HDR image with negative, zero, large and NaN pixels."""
    rng = np.random.RandomState(SEED)
    W, H = 36, 20  # W % 4 == 0: the reference's BMP padding write needs no padding
    img = (rng.exponential(0.8, (H, W, 3)) * rng.choice([0.1, 1.0, 10.0], (H, W, 1))).astype(np.float32)
    img[0, 0] = (-0.5, 0.0, 2.0)
    img[0, 1] = (np.nan, 0.25, 1.0)
    img[1, 2] = (1.0, 1.0, 1.0)
    out = {"img": img}
    for tag, limit, gamma in (("tm", 1.5, 0.0), ("gm", 0.0, 2.2), ("tmgm", 1.5, 2.2), ("tmgm2", 4.0, 1.8)):
        a = ref.tonemap_gamma(img, limit, gamma)
        b = orc.tonemap_gamma(img, limit, gamma)
        check_equal(f"resolve {tag}", np.nan_to_num(b, nan=-1), np.nan_to_num(a, nan=-1))
        out[tag] = a
    # int(NaN) in the exporters is undefined (x86 prints -2147483648 in the PPM,
    # Arm 0); the files are pinned on NaN-free pixels
    disp = np.where(np.isnan(out["tmgm"]), np.float32(0.5), out["tmgm"]).astype(np.float32)
    out["enc_in"] = disp
    for fmt in ("bmp", "ppm"):
        a = ref.encode(disp, fmt == "bmp")
        b = orc.encode(disp, fmt == "bmp")
        ok = a == b
        print(f"  {fmt}: {'byte-exact' if ok else 'MISMATCH'}")
        if not ok:
            raise SystemExit(f"oracle differs from the reference on {fmt}")
        out[fmt] = np.frombuffer(a, np.uint8)
    np.savez_compressed(os.path.join(OUT, "resolve.npz"), **out)


OBJ_DIR = os.path.join(OUT, "obj")


def _fmt(x, rng):
    """A float written in one of the notations operator>> accepts."""
    k = rng.randint(5)
    if k == 0:
        return f"{x:.6f}"
    if k == 1:
        return f"{x:.4e}"
    if k == 2:
        return f"{x:+.3E}"
    if k == 3:
        return repr(float(np.float32(x)))
    return f"{x:.2f}".replace("0.", ".", 1) if 0 < x < 1 else f"{x:.1f}"


def synthetic_obj_files():
    """Seeded OBJ / MTL texts exercising the importer's token rules: faces of
    3-6 vertices in v, v/vt, v//vn and v/vt/vn forms, runs of spaces, tabs,
    CRLF line ends, comments, ignored keys, 4-component vertices, -0.0,
    exponents; smoothing on and off; an 's off' that ends the import."""
    rng = np.random.RandomState(SEED)
    os.makedirs(OBJ_DIR, exist_ok=True)
    files = {}

    def obj_text(n_obj, crlf=False, s_off_after=None):
        L = ["# synthetic", "mtllib synthetic.mtl"]
        nv = nt = nn = 0
        for o in range(n_obj):
            L.append(f"o Object_{o}")
            L.append("g ignored_group")
            k = rng.randint(4, 9)
            for _ in range(k):
                xyz = rng.uniform(-3, 3, 3)
                if rng.rand() < 0.1:
                    xyz[rng.randint(3)] = -0.0
                extra = " 1.0" if rng.rand() < 0.1 else ""
                L.append("v " + " ".join(_fmt(c, rng) for c in xyz) + extra)
            nv += k
            for _ in range(k):
                L.append("vt " + " ".join(_fmt(c, rng) for c in rng.uniform(0, 1, 2)))
            nt += k
            for _ in range(k):
                n = rng.normal(size=3)
                n /= np.linalg.norm(n)
                L.append("vn " + " ".join(_fmt(c, rng) for c in n))
            nn += k
            L.append("usemtl " + ("Light" if o == 0 else "Grey"))
            L.append(f"s {int(rng.rand() < 0.5)}")
            for f in range(rng.randint(2, 6)):
                nvert = rng.randint(3, 7)
                ids = rng.choice(np.arange(nv - k + 1, nv + 1), nvert, replace=nvert > k)
                form = rng.randint(4)
                parts = []
                for i in ids:
                    t = rng.randint(nt - k + 1, nt + 1)
                    m = rng.randint(nn - k + 1, nn + 1)
                    parts.append([f"{i}", f"{i}/{t}", f"{i}//{m}", f"{i}/{t}/{m}"][form])
                sep = " " if rng.rand() < 0.7 else "   "
                lead = "" if rng.rand() < 0.7 else "  "
                trail = "" if rng.rand() < 0.7 else "  "
                L.append("f " + lead + sep.join(parts) + trail)
                if s_off_after is not None and o == s_off_after and f == 0:
                    L.append("s off")
            L.append("# end of object")
        return ("\r\n" if crlf else "\n").join(L) + "\n"

    files["basic.obj"] = obj_text(3)
    files["crlf.obj"] = obj_text(2, crlf=True)
    files["s_off.obj"] = obj_text(3, s_off_after=1)
    files["synthetic.mtl"] = "\n".join([
        "# materials", "newmtl Light", "Kd 0.780 0.780 0.780", "Ke 17 12 4", "Ns 10", "illum 2",
        "newmtl Grey", "Kd .5 .5 .5", "Ni 1.5", "Pr 0.25", "Pm 0.75", "Ps 0.1", "Pc 0.3", "Pcr 0.05",
        "aniso 0.2", "newmtl Default"]) + "\n"
    for name, text in files.items():
        with open(os.path.join(OBJ_DIR, name), "w", newline="") as f:
            f.write(text)
    return sorted(n for n in files if n.endswith(".obj"))


def obj_case(ref, ref_root):
    """RenderToy's OBJModelImporter / MTLImporter on the synthetic files
    (fixtures), and the native importer against it on the reference's own
    demo scenes (checked here only: those files are not copied)."""
    import rendertoy_gb300 as rt
    mtl = os.path.join(OBJ_DIR, "synthetic.mtl")
    out = {}
    for name in synthetic_obj_files():
        r = ref.obj_import(os.path.join(OBJ_DIR, name), mtl)
        tag = name[:-4]
        for k in ("verts", "norms", "uvs", "tri_mesh", "mesh_smooth", "mesh_counts", "mesh_tris", "materials"):
            out[f"{tag}_{k}"] = r[k]
        out[f"{tag}_mesh_names"] = np.array(r["mesh_names"])
        out[f"{tag}_material_names"] = np.array(r["material_names"])
        _obj_equal(rt.ObjModel(os.path.join(OBJ_DIR, name), mtl), r, name)
    np.savez_compressed(os.path.join(OUT, "obj.npz"), **out)
    for d in ("CornellBox", "SmoothShading", "WithOIDN", "Emissive"):
        dd = os.path.join(ref_root, "demo", d)
        if not os.path.isdir(dd):
            continue
        for f in sorted(os.listdir(dd)):
            if f.endswith(".obj"):
                p = os.path.join(dd, f)
                _obj_equal(rt.ObjModel(p), ref.obj_import(p), f"demo/{d}/{f}")


def _obj_equal(m, r, name):
    ok = (np.array_equal(bits(m.verts), bits(r["verts"] + np.float32(0.0)))
          and np.array_equal(bits(m.norms), bits(r["norms"])) and np.array_equal(bits(m.uvs), bits(r["uvs"]))
          and np.array_equal(m.tri_mesh, r["tri_mesh"]) and m.mesh_names == r["mesh_names"]
          and np.array_equal(np.array(m.mesh_smooth, np.uint8), r["mesh_smooth"])
          and np.array_equal(np.concatenate(m.mesh_tris) if m.mesh_tris else np.zeros(0, np.int32),
                             r["mesh_tris"])
          and m.material_names == r["material_names"] and np.array_equal(bits(m.materials), bits(r["materials"])))
    print(f"  {name}: {len(m.verts)} triangles, {len(m.mesh_names)} meshes: {'equal' if ok else 'MISMATCH'}")
    if not ok:
        raise SystemExit(f"native importer differs from the reference on {name}")


def write_obj_scene(sc, obj_path, mtl_path, cam_path):
    """A scene as OBJ + MTL text (one object per mesh, named m<i> after its
    material record; faces as triangles with v//vn) and its camera."""
    L, M = ["# scene"], ["# materials"]
    for k, m in enumerate(sc.mats):
        M += [f"newmtl mat{k}", "Kd " + " ".join(repr(float(x)) for x in m[0:3]),
              "Ke " + " ".join(repr(float(x)) for x in m[3:6]), f"Pr {float(m[6])!r}", f"Pm {float(m[7])!r}",
              f"Ps {float(m[11])!r}", f"Pc {float(m[13])!r}", f"Pcr {float(m[14])!r}", f"Ni {float(m[16])!r}"]
    nv = 0
    for mi in range(len(sc.mesh_mat)):
        ids = np.nonzero(sc.tri_mesh == mi)[0]
        L.append(f"o mat{int(sc.mesh_mat[mi])}")
        for t in ids:
            for k in range(3):
                L.append("v " + " ".join(repr(float(x)) for x in sc.verts[t, 3 * k:3 * k + 3]))
                L.append("vn " + " ".join(repr(float(x)) for x in sc.norms[t, 3 * k:3 * k + 3]))
        L.append(f"s {int(sc.mesh_smooth[mi])}")
        # faces in reverse so that Mesh::tris (prepend order) lists them forwards
        for j, t in reversed(list(enumerate(ids))):
            a = nv + 3 * j + 1
            L.append(f"f {a}//{a} {a + 1}//{a + 1} {a + 2}//{a + 2}")
        nv += 3 * len(ids)
    open(obj_path, "w").write("\n".join(L) + "\n")
    open(mtl_path, "w").write("\n".join(M) + "\n")
    np.asarray(sc.camera, np.float32).tofile(cam_path)


DEMO_OBJ = (64, 48, 128)  # W, H, spp


def demo_obj_case(ref_root):
    """tests/compat/demo_obj.cpp built against RenderToy's sources: its
    buffers and exported files on the mixed Cornell scene written as OBJ."""
    rdir = os.path.join(ROOT, "oracle", "_ref")
    exe = os.path.join(rdir, "demo_obj_ref")
    srcs = [os.path.join(ref_root, "src", s + ".cpp") for s in (
        "bvh", "object", "material", "rtmath", "surfacepoint", "world", "ray", "compositor",
        "exception", "procedural", "importer", "exporter", "renderer")]
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-include", "functional",
                           "-include", "vector", "-include", "cstdint", "-include", "optional",
                           "-include", "algorithm", "-I" + os.path.join(ref_root, "include"),
                           os.path.join(ROOT, "tests", "compat", "demo_obj.cpp"), *srcs, "-o", exe])
    d = os.path.join(rdir, "demo_obj")
    os.makedirs(d, exist_ok=True)
    sc = scenes.cornell_mixed()
    paths = [os.path.join(d, n) for n in ("scene.obj", "scene.mtl", "camera.bin")]
    write_obj_scene(sc, *paths)
    W, H, spp = DEMO_OBJ
    prefix = os.path.join(d, "ref")
    subprocess.check_call([exe, *paths, prefix, str(W), str(H), str(spp)])
    out = read_demo_output(prefix + ".bin")
    np.savez_compressed(os.path.join(OUT, "demo_obj.npz"), buffers=out, W=W, H=H, spp=spp,
                        bmp=np.frombuffer(open(prefix + "_normal.bmp", "rb").read(), np.uint8),
                        ppm=np.frombuffer(open(prefix + "_normal.ppm", "rb").read(), np.uint8))
    print(f"  demo_obj (reference build): {out.shape[0]} buffers")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None,
                    help="the RenderToy tree (default: the one oracle/Makefile reads, "
                         "RENDERTOY_SRC or the recipe's location)")
    ap.add_argument("--only", default="", help="regenerate one case: textures, resolve, obj")
    args = ap.parse_args()
    oracle_dir = os.path.join(ROOT, "oracle")
    if args.ref is None:
        args.ref = subprocess.check_output(["make", "-s", "-C", oracle_dir, "print-ref"], text=True).strip()
    if not os.path.isfile(os.path.join(args.ref, "src", "renderer.cpp")):
        raise SystemExit(f"no RenderToy tree at {args.ref!r}: pass --ref or set RENDERTOY_SRC")
    subprocess.check_call(["make", "-s", "-C", oracle_dir, f"RENDERTOY_SRC={args.ref}", "all", "ref"])
    ref, refo, orc = bind.load("ref"), bind.load("ref_orig"), bind.load("oracle")
    if args.only == "obj":
        obj_case(ref, args.ref)
        demo_obj_case(args.ref)
        return
    if args.only:
        {"textures": texture_case, "resolve": resolve_case}[args.only](ref, orc)
        return
    print("obj import:")
    obj_case(ref, args.ref)
    demo_obj_case(args.ref)
    print("resolve:")
    resolve_case(ref, orc)
    print("textures:")
    texture_case(ref, orc)
    print("scenes:")
    scene_case(ref, refo, orc, scenes.cornell_box(), 48, 40, "cornell")
    scene_case(ref, refo, orc, scenes.cornell_mixed(), 40, 32, "mixed")
    print("intersect:")
    intersect_case(ref, orc, scenes.cornell_mixed())
    print("bsdf:")
    bsdf_case(ref, orc)
    print("compositor:")
    compositor_case(ref, orc)
    print("rng:")
    rng_case(ref, orc)
    print("drop-in application:")
    demo_case(args.ref)
    print("written to", OUT)


if __name__ == "__main__":
    main()
