"""Pins the CPU oracle to the hand-derived known answers of tests/golden
(the reference itself has no tests or golden outputs to pin against)."""

from __future__ import annotations

import json
import os
from types import SimpleNamespace

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gold(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def kat_scene(dim, vmax=1.0, positions=None, normals=None, albedo=None, ls=None, ls_inverse=None, size=32,
              lights=()):
    f = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32))  # noqa: E731
    eye16 = np.eye(4, dtype=np.float32).reshape(16)
    return SimpleNamespace(
        dim=dim, levels=int(np.log2(dim)) + 1, vmax=vmax,
        positions=f(positions if positions is not None else np.zeros((0, 9))),
        normals=f(normals if normals is not None else np.zeros((0, 9))),
        albedo=f(albedo if albedo is not None else np.zeros((0, 3))),
        ntri=0 if positions is None else len(positions), lights=list(lights), shadow_size=(size, size),
        ls=f(ls if ls is not None else eye16), ls_inverse=f(ls_inverse if ls_inverse is not None else eye16),
        light_pos=f([0, 0, 0]), light_int=f([1, 1, 1]), eye=f([0, 0, 3]), gbuffer_size=(1, 1),
        cone=dict(diffuse=(16, np.radians(60), 1.0, 1.0, 0.5), specular=(32, np.radians(10), 1.7, 0.5, 0.1)))


def test_fp16_rounding_matches_ieee():
    g = gold("fp16.json")
    f32 = np.asarray(g["f32_bits"], dtype=np.uint32).view(np.float32)
    assert np.array_equal(O.f32_to_f16(f32), np.asarray(g["f16_bits"], dtype=np.uint16))
    # and the reverse conversion is exact
    h = np.asarray(g["f16_bits"], dtype=np.uint16)
    finite = np.isfinite(h.view(np.float16))
    assert np.array_equal(O.f16_to_f32(h)[finite], h.view(np.float16)[finite].astype(np.float32))


def test_voxel_mvp_matrices():
    g = gold("mvp.json")
    sc = kat_scene(g["dim"], g["vmax"])
    assert np.array_equal(O.voxel_mvp(sc), np.asarray(g["mvp"], dtype=np.float32))


def test_quad_voxelization_known_answer():
    g = gold("quad_voxel.json")
    sc = kat_scene(g["dim"], g["vmax"], g["positions"], g["normals"], g["albedo"])
    count, sums, total = O.voxelize(sc, np.ones(32 * 32, np.float32), lighting=0)
    N = g["dim"]
    idx = [(z * N + y) * N + x for x, y, z in g["voxels"]]
    expect = np.zeros(N ** 3, np.uint32)
    expect[idx] = g["count"]
    assert np.array_equal(count, expect)
    s = sums.reshape(6, -1)
    for k in range(6):
        e = np.zeros(N ** 3, np.uint32)
        e[idx] = g["sums"][k]
        assert np.array_equal(s[k], e), k
    assert total == g["total_fragments"]


def test_dominant_axis_tie_goes_to_z():
    g = gold("tie_axis.json")
    sc = kat_scene(g["dim"], g["vmax"], g["positions"], g["normals"], g["albedo"])
    count, _, total = O.voxelize(sc, np.ones(32 * 32, np.float32), lighting=0)
    assert total == g["total_fragments"] and not count.any()
    # the same triangle forced onto the x projection does produce fragments
    _, _, forced = O.voxelize(sc, np.ones(32 * 32, np.float32), lighting=0, axis_override=0)
    assert forced > 0


def test_shadow_map_known_answer():
    g = gold("shadow_quad.json")
    n = g["size"]
    sc = kat_scene(16, 1.0, g["positions"], np.zeros((2, 9)), np.zeros((2, 3)), ls=g["ls"], size=n)
    assert np.array_equal(O.render_shadowmap(sc), np.asarray(g["depth"], dtype=np.float32))


def test_inject_texel_corner_known_answer():
    g = gold("inject_plane.json")
    N, n = g["dim"], g["size"]
    sc = kat_scene(N, g["vmax"], ls=g["ls"], ls_inverse=g["ls_inverse"], size=n)
    color = np.tile(O.f32_to_f16(np.asarray(g["color"], np.float32)), N ** 3)
    normal = np.zeros_like(color)
    rad = np.zeros_like(color)
    O.inject(sc, np.full(n * n, g["depth"], np.float32), color, normal, rad)
    lit = rad.reshape(-1, 4)[:, 3] != 0
    expect = np.zeros(N ** 3, bool)
    expect[[(z * N + y) * N + x for x, y, z in g["lit_voxels"]]] = True
    assert np.array_equal(lit, expect)
    assert np.array_equal(rad.reshape(-1, 4)[lit], color.reshape(-1, 4)[lit])


def test_mip_point_known_answer():
    g = gold("mip_point.json")
    N, levels = g["dim"], g["levels"]
    chain = np.zeros(4 * O.chain_voxels(N, levels), np.uint16)
    x, y, z = g["voxel"]
    chain[4 * ((z * N + y) * N + x):][:4] = O.f32_to_f16(np.ones(4, np.float32))
    O.build_mips(N, levels, chain)
    offs = O.level_offsets(N, levels)
    for l in range(1, levels):
        S = N >> l
        lvl = O.f16_to_f32(chain[4 * offs[l]: 4 * (offs[l] + S ** 3)]).reshape(-1, 4)
        nz = np.flatnonzero(lvl[:, 0])
        assert len(nz) == len(g["expect"][l - 1])
        for xx, yy, zz, val in g["expect"][l - 1]:
            assert lvl[(zz * S + yy) * S + xx, 0] == val


def test_mip_of_constant_is_constant():
    N, levels = 32, 6
    chain = np.zeros(4 * O.chain_voxels(N, levels), np.uint16)
    chain[: 4 * N ** 3] = np.tile(O.f32_to_f16(np.asarray([0.3, 0.6, 0.1, 0.5], np.float32)), N ** 3)
    O.build_mips(N, levels, chain)
    assert np.array_equal(chain.reshape(-1, 4), np.tile(chain[:4], O.chain_voxels(N, levels)).reshape(-1, 4))


@pytest.mark.parametrize("precision", [32, 64])
def test_trace_constant_volume_closed_form(precision):
    g = gold("trace_const.json")
    N = g["dim"]
    sc = kat_scene(N)
    sc.gbuffer_size = (1, 1)
    chain = np.tile(O.f32_to_f16(np.full(4, g["value"], np.float32)), O.chain_voxels(N, sc.levels))
    gp = np.asarray(g["position"] + [1.0], np.float32)
    gn = np.asarray(g["normal"] + [0.0], np.float32)
    ga = np.ones(4, np.float32)
    irr, _, _, samples = O.trace(sc, chain, gp, gn, ga, precision=precision, enable_reflections=0)
    assert np.allclose(irr, g["irradiance"], rtol=0, atol=1e-6)
    assert samples == 6 * g["samples_per_cone"]
