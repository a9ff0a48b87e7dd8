"""The OBJ loader of the parity scenes (the reference reads its
resources/*.obj with tinyobjloader, src/Graphics/Mesh.cpp:41-190): faces of
every index form, fan triangulation of polygons, negative indices, zero
normals where the file has none, objects; and the reference's own meshes
when VCT_REFERENCE_RESOURCES names the reference's resources/ folder."""

from __future__ import annotations

import os

import numpy as np
import pytest

from vct_gb300 import scenes

REF_RESOURCES = os.environ.get("VCT_REFERENCE_RESOURCES", "")


def test_faces_of_every_index_form():
    text = """# a quad, a triangle with texture indices, a pentagon with negative indices
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 2 0 0
vt 0 0
vt 1 0
vt 1 1
vn 0 0 1
vn 0 0 -1
o first
f 1//1 2//1 3//1 4//1
f 1/1 2/2 5/3
o second
f -5/1/2 -4/2/2 -1/3/2 -3/1/2 -2/2/2
"""
    t, n, g = scenes.parse_obj(text)
    assert t.shape == (2 + 1 + 3, 3, 3)
    # quad (1,2,3,4) -> (1,2,3), (1,3,4)
    assert np.array_equal(t[0], [[0, 0, 0], [1, 0, 0], [1, 1, 0]])
    assert np.array_equal(t[1], [[0, 0, 0], [1, 1, 0], [0, 1, 0]])
    assert np.all(n[0] == [0, 0, 1]) and np.all(n[1] == [0, 0, 1])
    # v/vt faces carry no normal: zero, as the loader's zero-initialised vertex
    assert np.all(n[2] == 0)
    # pentagon -5 -4 -1 -3 -2 == 1 2 5 3 4, fanned around vertex 1
    assert np.array_equal(t[3], [[0, 0, 0], [1, 0, 0], [2, 0, 0]])
    assert np.array_equal(t[4], [[0, 0, 0], [2, 0, 0], [1, 1, 0]])
    assert np.array_equal(t[5], [[0, 0, 0], [1, 1, 0], [0, 1, 0]])
    assert np.all(n[3:] == [0, 0, -1])
    assert g.tolist() == [0, 0, 0, 1, 1, 1]


def test_generated_text_round_trip():
    tris = scenes.icosphere(2)
    t, n, g = scenes.parse_obj(scenes.obj_text(tris, tris))
    assert np.allclose(t, tris, atol=1e-8) and np.allclose(n, tris, atol=1e-8)
    # quads written from triangle pairs come back as the same pairs
    q = np.array([[[0, 0, 0], [1, 0, 0], [1, 1, 0]], [[0, 0, 0], [1, 1, 0], [0, 1, 0]]], dtype=np.float64)
    t2, _, _ = scenes.parse_obj(scenes.obj_text(q, quads=True))
    assert np.array_equal(t2, q)


def test_obj_scene_fits_the_volume():
    sc = scenes.obj_scene(scenes.obj_text(scenes.icosphere(3)), dim=32)
    mesh = sc.positions[10:].reshape(-1, 3)
    assert np.all(np.abs(mesh) <= 0.7 + 1e-6) and np.isclose(np.abs(mesh).max(), 0.7, atol=1e-5)
    assert sc.ntri == 10 + 1280 and sc.pv is not None


@pytest.mark.skipif(not os.path.isdir(REF_RESOURCES), reason="reference meshes not present")
@pytest.mark.parametrize("name,ntri,nobj", [("cube.obj", 12, 1), ("cubes.obj", 24, 2), ("sphere.obj", 720, 1),
                                            ("bunny.obj", 4968, 1)])
def test_reference_meshes(name, ntri, nobj):
    t, n, g = scenes.load_obj(os.path.join(REF_RESOURCES, name))
    assert t.shape == (ntri, 3, 3)
    assert int(g.max()) + 1 == nobj
    assert np.all(np.isfinite(t))
