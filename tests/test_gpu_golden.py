"""The hand-derived known answers of tests/golden, through the CUDA path and
the C ABI (volumes are seeded through zero-copy views of the context's
device memory where a stage is tested in isolation)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from helpers import read_chain, split_records, u16
from test_oracle_golden import gold, kat_scene
from vct_gb300 import _lib as L
from vct_gb300 import api

pytestmark = pytest.mark.gpu


def _tris(sc):
    import torch

    t = [torch.from_numpy(a).to("cuda:0") for a in (sc.positions, sc.normals, sc.albedo)]
    return t, api.triangles(*t)


def _ctx(sc, **over):
    ctx = api.Context(api.config_for(sc))
    p = api.scene_params(sc, **over)
    ctx.set_params(p)
    return ctx


def _shadow(sc, sm):
    return api.shadow_desc(sc, sm)


def test_quad_voxelization_known_answer():
    import torch

    g = gold("quad_voxel.json")
    sc = kat_scene(g["dim"], g["vmax"], g["positions"], g["normals"], g["albedo"])
    keep, tris = _tris(sc)
    sm = torch.ones(32 * 32, device="cuda:0")
    with _ctx(sc, voxelize_lighting=0) as ctx:
        ctx.voxelize_accumulate(tris, api.light_array([]), _shadow(sc, sm), sc.eye)
        torch.cuda.synchronize()
        count, sums, occ, _ = split_records(*ctx.read_accumulators())
        ctx.normalize()
        st = ctx.stats()
    N = g["dim"]
    idx = [(z * N + y) * N + x for x, y, z in g["voxels"]]
    expect = np.zeros(N ** 3, np.uint32)
    expect[idx] = 1
    assert np.array_equal(count, expect) and np.array_equal(occ, expect > 0)
    s = sums.reshape(6, -1)
    for k in range(6):
        assert (s[k][idx] == g["sums"][k]).all() and s[k].sum() == g["sums"][k] * len(idx)
    assert st["total_voxel_fragments"] == g["total_fragments"] and st["unique_voxels"] == len(idx)


def test_shadow_map_known_answer():
    import torch

    g = gold("shadow_quad.json")
    n = g["size"]
    sc = kat_scene(16, 1.0, g["positions"], np.zeros((2, 9)), np.zeros((2, 3)), ls=g["ls"], size=n)
    keep, tris = _tris(sc)
    out = torch.empty(n * n, device="cuda:0")
    api.render_shadowmap(tris, sc, out)
    assert np.array_equal(out.cpu().numpy(), np.asarray(g["depth"], np.float32))


def test_inject_texel_corner_known_answer():
    import torch

    g = gold("inject_plane.json")
    N, n = g["dim"], g["size"]
    sc = kat_scene(N, g["vmax"], ls=g["ls"], ls_inverse=g["ls_inverse"], size=n)
    sm = torch.full((n * n,), g["depth"], device="cuda:0")
    color = np.tile(O.f32_to_f16(np.asarray(g["color"], np.float32)), N ** 3)
    with _ctx(sc) as ctx:
        ptr, _ = ctx.volume_ptr(L.VCT_VOLUME_COLOR, 0)
        api.device_view(ptr, (N ** 3 * 4,), "<i2").copy_(torch.from_numpy(color.view(np.int16)))
        ctx.inject(_shadow(sc, sm), sc.eye)
        torch.cuda.synchronize()
        rad = u16(ctx.read_volume(L.VCT_VOLUME_RADIANCE, 0)).reshape(-1, 4)
    expect = np.zeros(N ** 3, bool)
    expect[[(z * N + y) * N + x for x, y, z in g["lit_voxels"]]] = True
    assert np.array_equal(rad[:, 3] != 0, expect)
    assert np.array_equal(rad[expect], color.reshape(-1, 4)[expect])


def test_mip_point_known_answer():
    import torch

    g = gold("mip_point.json")
    N, levels = g["dim"], g["levels"]
    sc = kat_scene(N)
    with _ctx(sc) as ctx:
        ptr, _ = ctx.volume_ptr(L.VCT_VOLUME_RADIANCE, 0)
        l0 = np.zeros(4 * N ** 3, np.uint16)
        x, y, z = g["voxel"]
        l0[4 * ((z * N + y) * N + x):][:4] = O.f32_to_f16(np.ones(4, np.float32))
        api.device_view(ptr, (N ** 3 * 4,), "<i2").copy_(torch.from_numpy(l0.view(np.int16)))
        ctx.build_mips()
        torch.cuda.synchronize()
        for l in range(1, levels):
            S = N >> l
            lvl = O.f16_to_f32(u16(ctx.read_volume(L.VCT_VOLUME_RADIANCE, l))).reshape(-1, 4)
            assert np.count_nonzero(lvl[:, 0]) == len(g["expect"][l - 1])
            for xx, yy, zz, val in g["expect"][l - 1]:
                assert lvl[(zz * S + yy) * S + xx, 0] == val


@pytest.mark.parametrize("hardware", [False, True])
def test_trace_constant_volume_closed_form(hardware):
    import torch

    g = gold("trace_const.json")
    N = g["dim"]
    sc = kat_scene(N)
    with _ctx(sc, enable_reflections=0, trace_filter=int(hardware)) as ctx:
        ptr, _ = ctx.volume_ptr(L.VCT_VOLUME_RADIANCE, 0)
        val = O.f32_to_f16(np.full(4, g["value"], np.float32))
        api.device_view(ptr, (N ** 3 * 4,), "<i2").copy_(torch.from_numpy(np.tile(val, N ** 3).view(np.int16)))
        ctx.build_mips()  # mips of a constant are the constant, exactly
        chain = read_chain(ctx)
        assert np.array_equal(chain, np.tile(val, len(chain) // 4))
        gp = torch.tensor(g["position"] + [1.0], device="cuda:0")
        gn = torch.tensor(g["normal"] + [0.0], device="cuda:0")
        ga = torch.ones(4, device="cuda:0")
        irr = torch.zeros(4, device="cuda:0")
        samples = torch.zeros(1, dtype=torch.int64, device="cuda:0")
        ctx.trace(api.gbuffer(gp, gn, ga, 1, 1), sc.eye, api.trace_out(irradiance=irr, samples=samples))
        torch.cuda.synchronize()
    assert np.allclose(irr.cpu().numpy(), g["irradiance"], rtol=0, atol=1e-6)
    assert int(samples.item()) == 6 * g["samples_per_cone"]
