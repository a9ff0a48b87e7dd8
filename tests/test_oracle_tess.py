"""The oracle's tessellation voxeliser (simpleTesselated.vert,
testTesselation.tesc/.tese, and GL's triangle primitive generator in point
mode with equal spacing, OpenGL 4.6 section 11.2.2.1): hand-computed levels of
the control shader, the point set's counts and geometry against the spec's
construction, and the perspective warp (voxelizeTesselationWarp)."""

from __future__ import annotations

import itertools

import numpy as np
import pytest

import oracle as O
from vct_gb300 import scenes


def _inner_points(n: int) -> int:
    """Concentric inner rings of an inner level n: ring k has n - 2k segments."""
    total = 0
    for k in range(1, n // 2 + 1):
        q = n - 2 * k
        total += 3 * q if q > 0 else 1
    return total


@pytest.mark.parametrize("levels", [(1, 1, 1, 1), (2, 1, 1, 1), (2, 3, 1, 2), (3, 2, 2, 2), (4, 4, 4, 4),
                                    (5, 5, 6, 3), (6, 1, 7, 2), (7, 7, 7, 7), (64, 64, 64, 64), (63, 1, 64, 2)])
def test_point_set_counts_and_geometry(levels):
    n, m0, m1, m2 = levels
    c = O.tess_coords(levels).astype(np.float64)
    assert len(c) == m0 + m1 + m2 + _inner_points(n)
    assert np.all(c >= 0) and np.allclose(c.sum(1), 1, atol=1e-6)
    assert len(np.unique(np.round(c, 6), axis=0)) == len(c)  # point mode: every vertex once
    # corners, then the inner points of the u = 0, v = 0 and w = 0 edges at j / m
    assert np.array_equal(c[:3], np.eye(3))
    o = 3
    for axis, m in ((0, m0), (1, m1), (2, m2)):
        e = c[o:o + m - 1]
        assert np.all(e[:, axis] == 0)
        other = (axis + 2) % 3  # the coordinate that grows along the edge
        assert np.allclose(np.sort(e[:, other]), np.arange(1, m) / m, atol=1e-6)
        o += m - 1
    # inner ring k: min(u, v, w) = 2k / (3n), 3 (n - 2k) points (the centre when n - 2k = 0)
    inner = c[o:]
    mins = inner.min(1)
    for k in range(1, n // 2 + 1):
        q = n - 2 * k
        on = np.isclose(mins, 2 * k / (3 * n), atol=1e-6)
        assert on.sum() == (3 * q if q > 0 else 1), (k, q)
    if n % 2 == 0 and n >= 2:
        assert np.allclose(inner[-1], 1 / 3)


def test_inner_corner_is_the_perpendicular_construction():
    """In the equilateral domain the first inner ring's corner near vertex 0
    lies on the perpendiculars to edges 0-1 and 0-2 through the subdivision
    points at distance 1/n from vertex 0 (OpenGL 4.6, 11.2.2.1)."""
    P = np.array([[0.0, 0.0], [1.0, 0.0], [0.5, np.sqrt(3) / 2]])  # vertices 0, 1, 2, side 1
    for n in (3, 4, 5, 8, 17, 64):
        c = O.tess_coords((n, 1, 1, 1)).astype(np.float64)[3:]
        corner = c[np.argmax(c[:, 0])]  # the ring-1 point nearest vertex 0
        x = corner @ P
        for edge in (P[1] - P[0], P[2] - P[0]):
            along = (x - P[0]) @ edge  # unit edges: projection length
            assert abs(along - 1.0 / n) < 1e-6, (n, along)
        # ring 1's points keep the subdivision spacing 1/n along its edges
        ring = c[np.isclose(c.min(1), 2 / (3 * n), atol=1e-6)] @ P
        d = np.sort(np.linalg.norm(ring[:, None] - ring[None], axis=-1), axis=1)[:, 1]
        if n > 3:
            assert np.allclose(d, 1.0 / n, atol=1e-5)


def _vol(dim):
    sc = scenes.tiny(seed=0)
    sc.dim = dim
    return sc


def test_control_shader_levels_known_answers():
    sc = _vol(16)  # volume [-1, 1]^3, voxel size 0.125
    # right triangle a=(0,0,0) b=(0.55,0,0) c=(0,0.3,0):
    #   |C| = |b-a| = 0.55 -> 4.4, |A| = |c-b| = 0.62650 -> 5.012, |B| = |c-a| = 0.3 -> 2.4 (in voxels);
    #   area 0.0825, altitudes 0.2634, 0.55, 0.3 -> inner 0.55 / 0.125 = 4.4;
    #   rounded up: inner 5, outer[0] = C 5, outer[1] = A 6, outer[2] = B 3
    tri = [0, 0, 0, 0.55, 0, 0, 0, 0.3, 0]
    assert O.tess_levels(sc, tri) == (5, 5, 6, 3)
    assert len(O.tess_coords((5, 5, 6, 3))) == 26
    # all three vertices in voxel (8, 8, 8): the control shader sets the levels to 0 (discarded)
    assert O.tess_levels(sc, [0.01, 0.01, 0.01, 0.1, 0.02, 0.03, 0.05, 0.1, 0.11]) is None
    # a sliver: short edge C = b - a of 0.05 (0.4 voxels -> 1) and long edges of 1.2 (9.6 voxels -> 10),
    # inner 9.6 -> 10; outer[0] is the short edge C
    assert O.tess_levels(sc, [0, -0.6, 0.3, 0.05, -0.6, 0.3, 0.025, 0.6, 0.3]) == (10, 1, 10, 10)
    # levels above GL_MAX_TESS_GEN_LEVEL are clamped: a 1.9-long edge in a 256^3 grid is 243 voxels
    big = _vol(256)
    lv = O.tess_levels(big, [-0.95, -0.95, 0, 0.95, -0.95, 0, -0.95, 0.95, 0])
    assert lv == (64, 64, 64, 64)
    assert O.tess_levels(big, [-0.95, -0.95, 0, 0.95, -0.95, 0, -0.95, 0.95, 0], max_level=32.0) == (32, 32, 32, 32)
    # a level of exactly one everywhere but one edge: inner 1 + epsilon -> 2
    lv = O.tess_levels(sc, [0, 0, 0, 0.2, 0, 0, 0, 0.1, 0])
    assert lv[0] >= 2


def test_voxelize_tess_counts_and_threads():
    sc = scenes.tiny(seed=2, dim=32)
    c1, s1, t1 = O.voxelize_tess(sc, nthreads=1)
    c4, s4, t4 = O.voxelize_tess(sc, nthreads=4)
    assert t1 == t4 and np.array_equal(c1, c4) and np.array_equal(s1, s4)
    # every generated point of a non-discarded patch is counted
    expect = 0
    for tri in sc.positions:
        lv = O.tess_levels(sc, tri)
        if lv is not None:
            expect += len(O.tess_coords(lv))
    assert t1 == expect
    assert c1.sum() <= t1 and c1.sum() > 0.9 * t1  # the boxes lie inside the volume
    # unlit: colour sums are the albedo's 16-bit fixed point times the count
    N3 = 32 ** 3
    occ = np.nonzero(c1)[0]
    single = occ[c1[occ] == 1]
    assert np.all(s1[:N3][single] <= 65535)


def test_perspective_warp_with_identity_pv_is_the_linear_map():
    """voxelTesselationWarpedPosition with pv = identity is p * 0.5 + 0.5,
    which for the volume [-1, 1]^3 is voxelLinearPosition exactly."""
    sc = scenes.tiny(seed=4, dim=32)
    sc.pv = np.eye(4, dtype=np.float32).reshape(16)
    lin = O.voxelize_tess(sc)
    per = O.voxelize_tess(sc, warp=O.warp(sc, 3))
    assert lin[2] == per[2]
    assert np.array_equal(lin[0], per[0]) and np.array_equal(lin[1], per[1])


def test_perspective_warp_drops_points_behind_the_camera():
    sc = scenes.tiny(seed=4, dim=32)
    # the scene's pv: camera at sc.eye looking at the origin, near 1, far 20
    w = O.warp(sc, 3)
    c, s, t = O.voxelize_tess(sc, warp=w)
    assert c.sum() > 0
    # moving every triangle behind the camera leaves nothing on the grid
    back = sc.positions.reshape(-1, 3, 3) + 4.0 * (sc.eye / np.linalg.norm(sc.eye))[None, None]
    c2, _, t2 = O.voxelize_tess(sc, warp=w, positions=back.reshape(-1, 9).astype(np.float32))
    assert t2 == t and c2.sum() == 0


def test_perspective_warp_froxel_grid():
    """The projected grid: a point at the camera's target lands in the
    centre column of the froxel grid, and nearer points get smaller depth."""
    sc = scenes.tiny(seed=4, dim=64)
    w = O.warp(sc, 3)
    eye = sc.eye.astype(np.float64)
    fwd = -eye / np.linalg.norm(eye)
    tri = []
    for d in (1.5, 2.0, 2.5):
        p = eye + d * fwd
        # a sliver along the view ray: it spans several linear voxels (not discarded) but one froxel column
        tri.append(np.concatenate([p, p + [0.001, 0, 0], p + 0.1 * fwd]))
    pos = np.array(tri, dtype=np.float32)
    nrm = np.tile(np.array([0, 0, 1, 0, 0, 1, 0, 0, 1], np.float32), (3, 1))
    alb = np.full((3, 3), 0.5, np.float32)
    zs = []
    for k in range(3):
        c, _, _ = O.voxelize_tess(sc, warp=w, positions=pos[k:k + 1], normals=nrm[k:k + 1], albedo=alb[k:k + 1])
        v = np.nonzero(c)[0]
        assert len(v) > 0
        x, y, z = v % 64, (v // 64) % 64, v // 4096
        assert np.all(np.abs(x - 32) <= 2) and np.all(np.abs(y - 32) <= 2)
        zs.append(z.min())
    assert zs[0] < zs[1] < zs[2]


def test_all_small_level_combinations():
    for lv in itertools.product(range(1, 7), repeat=4):
        n = lv[0]
        if n == 1 and max(lv[1:]) > 1:
            continue  # never produced: 1 + epsilon rounds to 2
        c = O.tess_coords(lv)
        assert len(c) == sum(lv[1:]) + _inner_points(n)
        assert len(np.unique(np.round(c.astype(np.float64), 6), axis=0)) == len(c)
