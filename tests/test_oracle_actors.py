"""Known answers of the rigid-actor transform (voxelize.vert's model matrix
for positions, mat3(transpose(inverse(model))) for normals; src/Actor.h):
a non-uniform scale, a rotation about y with a translation, and triangles
outside every actor range left as they are."""

from __future__ import annotations

import numpy as np

import oracle as O


def colmajor(m):
    return np.ascontiguousarray(np.asarray(m, dtype=np.float64).T.reshape(16), dtype=np.float32)


def test_normal_matrix_of_a_nonuniform_scale():
    m = np.diag([2.0, 1.0, 4.0, 1.0])
    m[:3, 3] = [5.0, -1.0, 0.5]  # translation does not reach the normals
    nm = O.normal_matrix(colmajor(m)).reshape(3, 3).T  # column-major 3x3 -> row-major
    assert np.allclose(nm, np.diag([0.5, 1.0, 0.25]), rtol=1e-7)


def test_rotation_and_translation_of_positions_and_normals():
    # 90 degrees about +y: x -> -z, z -> x; then translate by (1, 2, 3)
    m = np.array([[0.0, 0.0, 1.0, 1.0], [0.0, 1.0, 0.0, 2.0], [-1.0, 0.0, 0.0, 3.0], [0.0, 0.0, 0.0, 1.0]])
    pos = np.array([[1, 0, 0, 0, 1, 0, 0, 0, 1], [9, 9, 9, 9, 9, 9, 9, 9, 9]], np.float32)
    nrm = np.array([[1, 0, 0, 0, 1, 0, 0, 0, 1], [1, 0, 0, 1, 0, 0, 1, 0, 0]], np.float32)
    p, n = O.transform_actors(pos, nrm, [0], [1], colmajor(m))
    assert np.allclose(p[0], [1, 2, 2, 1, 3, 3, 2, 2, 3], atol=1e-6)
    assert np.allclose(n[0], [0, 0, -1, 0, 1, 0, 1, 0, 0], atol=1e-6)
    # the second triangle is outside every actor's range
    assert np.array_equal(p[1], pos[1]) and np.array_equal(n[1], nrm[1])
