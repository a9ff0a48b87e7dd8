"""Known answers of the oracle's voxel warping (no GPU): the 32^3 warp map of
empty, full and half-occupied grids in closed form (Application.cpp:346-371,
generateWarpmap.frag), and the analytic warp's fixed points (common.glsl)."""

from __future__ import annotations

import ctypes as C

import numpy as np

import oracle as O

D = 32


def centre_unorm(i):
    return np.rint((i + 0.5) / D * 65535).astype(np.uint16)


def test_empty_and_full_grids_give_the_identity():
    idx = np.arange(D)
    for occ in (np.zeros(D ** 3, bool), np.ones(D ** 3, bool)):
        m = O.warpmap(occ).reshape(D, D, D, 4)  # z, y, x, c
        assert np.array_equal(m[..., 0], np.broadcast_to(centre_unorm(idx)[None, None, :], (D, D, D)))
        assert np.array_equal(m[..., 1], np.broadcast_to(centre_unorm(idx)[None, :, None], (D, D, D)))
        assert np.array_equal(m[..., 2], np.broadcast_to(centre_unorm(idx)[:, None, None], (D, D, D)))
    full = O.warpmap(np.ones(D ** 3, bool)).reshape(D, D, D, 4)
    # packCellInfo: totals of 32 wrap to 0 in 5 bits, occupied bit set
    assert np.all(full[..., 3] == 1 << 15)


def test_half_occupied_rows():
    occ = np.zeros((D, D, D), bool)  # z, y, x
    occ[:, :, :16] = True            # every x row: cells 0..15 occupied
    m = O.warpmap(occ).reshape(D, D, D, 4)
    # 16 of 32 occupied: h = 2 gives l = 0 < 0.5, so l = 0.5 and h = (32 - 0.5 * 16) / 16 = 1.5
    x = np.arange(D, dtype=np.float64)
    want = np.where(x < 16, (1.5 * x + 0.75) / D, (0.5 * (x - 16) + 1.5 * 16 + 0.25) / D)
    assert np.array_equal(m[0, 0, :, 0], np.rint(want * 65535).astype(np.uint16))
    # along y and z each row is all occupied or all empty: identity
    assert np.array_equal(m[:, :, 3, 1], np.broadcast_to(centre_unorm(np.arange(D))[None, :], (D, D)))
    # totals: 16 along x, 32 -> 0 along y and z for occupied cells, 0 for empty
    assert m[0, 0, 0, 3] == (16 | (1 << 15)) and m[0, 0, 20, 3] == 16


def test_low_resolution_floor():
    occ = np.zeros((D, D, D), bool)
    occ[0, 0, :4] = True  # 4 occupied of 32 in one x row: l = (32 - 2 * 4) / 28 = 6/7, above the floor
    m = O.warpmap(occ).reshape(D, D, D, 4)
    l = np.float32(np.float16(np.float32(24) / np.float32(28)))
    x = np.arange(D, dtype=np.float32)
    prev = np.minimum(x, 4)
    occd = x < 4
    res = np.where(occd, np.float32(2), l)
    pv = np.where(occd, x, prev)
    offset = l * (x - pv) + np.float32(2) * pv
    w = (offset + np.float32(0.5) * res) / np.float32(D)
    assert np.array_equal(m[0, 0, :, 0], np.rint(np.clip(w, 0, 1) * np.float32(65535)).astype(np.uint16))


def test_warped_voxelisation_with_an_identity_map_keeps_the_pixel_columns():
    """An empty occupancy grid gives the identity map (cell centres): a
    fragment's x and y then land in the voxel of its pixel centre, so the
    warped and unwarped voxelisations of a face-on quad agree in x and y."""
    from vct_gb300 import scenes

    sc = scenes.tiny(dim=16)
    quad = np.array([[-0.9, -0.9, 0.3, 0.9, -0.9, 0.3, 0.9, 0.9, 0.3],
                     [-0.9, -0.9, 0.3, 0.9, 0.9, 0.3, -0.9, 0.9, 0.3]], np.float32)
    nrm = np.tile(np.array([0, 0, 1], np.float32), (2, 3))
    alb = np.full((2, 3), 0.5, np.float32)
    sm = np.ones(sc.shadow_size[0] * sc.shadow_size[1], np.float32)
    plain, _, t0 = O.voxelize(sc, sm, lighting=0, positions=quad, normals=nrm, albedo=alb)
    w = O.warp(sc, 2, O.warpmap(np.zeros(D ** 3, bool)))
    warped, _, t1 = O.voxelize(sc, sm, lighting=0, positions=quad, normals=nrm, albedo=alb, warp=w)
    assert t0 == t1 > 0
    N = sc.dim
    pz, py, px = np.nonzero(plain.reshape(N, N, N) > 0)
    wz, wy, wx = np.nonzero(warped.reshape(N, N, N) > 0)
    assert sorted(zip(px, py)) == sorted(zip(wx, wy))
    assert abs(int(np.median(wz)) - int(np.median(pz))) <= 1
