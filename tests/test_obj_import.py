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
