"""Voxel warping against the oracle: the 32^3 warp map (warpTexture) and the
analytic warp about the eye (warpVoxels) through voxelisation, injection,
the mip chain and the cone trace.  Integer and binary16 results are
bit-exact; irradiance within the trace tolerances."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from helpers import GpuScene, read_chain, rel_l2, rgb, split_records, u16
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[L.VCT_WARP_ANALYTIC, L.VCT_WARP_TEXTURE], ids=["analytic", "texture"])
def warped(request):
    import torch

    mode = request.param
    if mode == L.VCT_WARP_ANALYTIC:
        # voxelWarp magnifies the volume around the eye and pushes what lies
        # farther than ~0.42 of the extent out of the grid: boxes near the
        # centre, warped (and reflected) about the volume's centre
        sc = scenes.tiny(seed=3, dim=64, shadow=512, gbuffer=(320, 180), n_boxes=12)
        g = GpuScene(sc)  # shadow map and G-buffer from the scene's camera
        sc.eye = np.array([0.0, 0.0, 0.0], np.float32)
    else:
        sc = scenes.cornell(seed=6)
        g = GpuScene(sc)
    sm, gbuf = g.host_inputs()
    ref = O.frame(sc, shadowmap=sm, gbuf=gbuf, warp_mode=mode, nthreads=8)
    ref64 = O.trace(sc, ref["chain"], *gbuf, precision=64, want=("irr",), warp=ref["warp"], nthreads=8)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc, warp_mode=mode))
    ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, sc.eye)
    torch.cuda.synchronize()
    cnt, sums, occ, _ = split_records(*ctx.read_accumulators())
    wmap = ctx.read_warpmap().cpu().numpy().view(np.uint16) if mode == L.VCT_WARP_TEXTURE else None
    ctx.normalize()
    ctx.inject(g.shadow, sc.eye)
    ctx.build_mips()
    irr, spec, col, samples = g.new_outputs()
    ctx.trace(g.gb, sc.eye, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    stages = dict(count=cnt, sums=sums, occ=occ, wmap=wmap, chain=read_chain(ctx), irr=irr.cpu().numpy(),
                  stats=ctx.stats())
    # the fused frame on a second context
    ctx2 = api.Context(api.config_for(sc))
    ctx2.set_params(api.scene_params(sc, warp_mode=mode))
    irr2, spec2, col2, samples2 = g.new_outputs()
    ctx2.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr2, spec2, col2, samples2))
    torch.cuda.synchronize()
    fused = dict(chain=read_chain(ctx2), irr=irr2.cpu().numpy(), stats=ctx2.stats())
    # the fused frame with the hybrid sampler, on a third context
    ctx3 = api.Context(api.config_for(sc))
    ctx3.set_params(api.scene_params(sc, warp_mode=mode, trace_filter=L.VCT_FILTER_HYBRID))
    irr3, spec3, col3, samples3 = g.new_outputs()
    ctx3.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr3, spec3, col3, samples3))
    torch.cuda.synchronize()
    fused["hybrid_irr"] = irr3.cpu().numpy()
    fused["hybrid_chain"] = read_chain(ctx3)
    return mode, sc, ref, ref64, stages, fused


def test_warpmap_bitexact(warped):
    mode, sc, ref, _, st, _ = warped
    if mode != L.VCT_WARP_TEXTURE:
        pytest.skip("analytic warp has no map")
    assert np.array_equal(st["wmap"], ref["warpmap"])
    # the map is not the identity for this scene
    D = 32
    idx = np.arange(D)
    ident = np.rint((idx + 0.5) / D * 65535).astype(np.uint16)
    assert not np.array_equal(st["wmap"].reshape(D, D, D, 4)[..., 0], np.broadcast_to(ident, (D, D, D)))


def test_warpmap_bitexact_turned_slivers():
    """The map's occupancy pass on thin cylinder slivers turned off the grid axes
    (the dynamic scene's actors moved to t = 1.3), boxes and columns, plus a
    floor quad whose triangles span the whole 32^2 viewport: small bounding
    boxes are walked by their own thread, the large ones by the warp."""
    import copy

    import torch

    sc, actors = scenes.dynamic_scene(seed=2, n_actors=8, dim=64, shadow=512, gbuffer=(160, 90), static_boxes=200,
                                      static_cyl=6)
    pos = sc.positions.reshape(-1, 3, 3).astype(np.float64)
    nrm = sc.normals.reshape(-1, 3, 3).astype(np.float64)
    for first, count, M in actors.models(1.3):
        pos[first:first + count] = pos[first:first + count] @ M[:3, :3].T + M[:3, 3]
        nrm[first:first + count] = nrm[first:first + count] @ M[:3, :3].T
    f = 0.97
    floor = np.array([[[-f, -f, -f], [-f, -f, f], [f, -f, f]], [[-f, -f, -f], [f, -f, f], [f, -f, -f]]])
    sc2 = copy.copy(sc)
    sc2.positions = np.ascontiguousarray(np.concatenate([pos, floor]).reshape(-1, 9), dtype=np.float32)
    sc2.normals = np.ascontiguousarray(
        np.concatenate([nrm, np.broadcast_to([0.0, 1.0, 0.0], (2, 3, 3))]).reshape(-1, 9), dtype=np.float32)
    sc2.albedo = np.ascontiguousarray(np.concatenate([sc.albedo, np.full((2, 3), 0.5)]), dtype=np.float32)
    g = GpuScene(sc2)
    sm, _ = g.host_inputs()
    occ = O.warp_occupancy(sc2, sm, nthreads=8)
    assert 0 < occ.sum() < occ.size
    ctx = api.Context(api.config_for(sc2))
    ctx.set_params(api.scene_params(sc2, warp_mode=L.VCT_WARP_TEXTURE))
    ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, sc2.eye)
    torch.cuda.synchronize()
    wmap = ctx.read_warpmap().cpu().numpy().view(np.uint16)
    assert np.array_equal(wmap, O.warpmap(occ))


def test_warped_accumulators_bitexact(warped):
    mode, sc, ref, _, st, _ = warped
    assert ref["count"].sum() > 100
    assert np.array_equal(st["count"], ref["count"])
    assert np.array_equal(st["sums"], ref["sums"])
    assert np.array_equal(st["occ"], ref["count"] > 0)
    # warping moved voxels relative to the plain voxelisation
    plain, _, _ = O.voxelize(sc, O.render_shadowmap(sc), nthreads=8)
    assert not np.array_equal(plain > 0, ref["count"] > 0)


def test_warped_chain_bitexact_stage_and_fused(warped):
    mode, sc, ref, _, st, fused = warped
    assert np.array_equal(st["chain"], ref["chain"])
    assert np.array_equal(fused["chain"], ref["chain"])
    for k in ("total_voxel_fragments", "unique_voxels", "max_fragments_per_voxel"):
        assert st["stats"][k] == ref["stats"][k] == fused["stats"][k], k


def test_warped_trace_matches_oracles(warped):
    mode, sc, ref, ref64, st, fused = warped
    irr = rgb(st["irr"])
    assert np.abs(irr).sum() > 0
    assert rel_l2(irr, rgb(ref["irradiance"])) <= 1e-5
    e64 = rel_l2(irr, rgb(ref64[0]))
    print(f"warp mode {mode}: irradiance rel L2 vs fp64 {e64:.2e}")
    assert e64 <= 1e-3
    assert np.array_equal(st["irr"].view(np.uint32), fused["irr"].view(np.uint32))


def test_warped_hybrid_sampler_within_bar(warped):
    """The hybrid sampler (the heavier-weighted level of each sample exact, the
    other by the texture units) on the warped chain: held to the 1e-3 fp64 bar,
    and its frame's chain equals the oracle's."""
    mode, sc, ref, ref64, st, fused = warped
    assert np.array_equal(fused["hybrid_chain"], ref["chain"])
    e64 = rel_l2(rgb(fused["hybrid_irr"]), rgb(ref64[0]))
    print(f"warp mode {mode}: hybrid irradiance rel L2 vs fp64 {e64:.2e}")
    assert e64 <= 1e-3


_A, _T, _N = L.VCT_WARP_ANALYTIC, L.VCT_WARP_TEXTURE, L.VCT_WARP_NONE


@pytest.mark.parametrize("modes", [(_A, _A, _A), (_T, _T, _T), (_T, _N, _A)], ids=["analytic", "texture", "mixed"])
def test_batch_with_warps_equals_single_frames(modes):
    """Batched frames with warped scenes: the analytic warp about each eye, the
    texture warp (each scene's occupancy pass and map built inside the batched
    frame), or a mix; chains, maps and irradiance equal single frames, bit for
    bit."""
    import torch

    scs = [scenes.batch_scene(seed=5, index=i) for i in range(3)]
    gs = [GpuScene(sc) for sc in scs]
    for sc in scs:
        sc.eye = np.array([0.0, 0.0, 0.0], np.float32)  # warp about the centre
    ref = []
    for sc, g, mode in zip(scs, gs, modes):
        ctx = api.Context(api.config_for(sc))
        ctx.set_params(api.scene_params(sc, warp_mode=mode))
        o = g.new_outputs()
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
        torch.cuda.synchronize()
        wmap = ctx.read_warpmap().cpu().numpy() if mode == _T else None
        ref.append((read_chain(ctx), o[0].cpu().numpy(), wmap))
    b = api.Batch([api.config_for(sc) for sc in scs])
    for i, (sc, mode) in enumerate(zip(scs, modes)):
        b.set_params(api.scene_params(sc, warp_mode=mode), i)
    outs = [g.new_outputs() for g in gs]
    for _ in range(2):  # the second frame checks that the occupancy masks were cleared
        b.frame([api.scene_desc(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
                 for sc, g, o in zip(scs, gs, outs)])
    torch.cuda.synchronize()
    for i, mode in enumerate(modes):
        assert np.array_equal(read_chain(b.scenes[i]), ref[i][0])
        assert np.array_equal(outs[i][0].cpu().numpy().view(np.uint32), ref[i][1].view(np.uint32))
        if mode == _T:
            assert np.array_equal(b.scenes[i].read_warpmap().cpu().numpy(), ref[i][2])
