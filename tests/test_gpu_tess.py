"""The tessellation voxeliser (testTesselation.tesc/.tese) and the
perspective warp (voxelizeTesselationWarp) against the oracle: accumulators
bit-exact with and without the warp, sums past 2^32 (more than 65,536 points
in one voxel) exact through the carry table, the whole frame with either
voxeliser under the perspective warp (volumes bit-exact, irradiance within
the trace tolerances), and the batch's refusal."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from helpers import GpuScene, read_chain, rel_l2, rgb, split_records
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu

CASES = {
    # walls span the grid (levels near the 64 limit), a sphere of small triangles (many discarded)
    "cornell": lambda: scenes.cornell(seed=2),
    # boxes and slivers of the large frame's family: columns of 256 segments put many points in one voxel
    "family": lambda: scenes.large_family(seed=3, dim=128, shadow=1024, gbuffer=(320, 180), n_boxes=512, n_cyl=8,
                                          cyl_segments=256),
}


@pytest.fixture(scope="module", params=[(c, w) for c in CASES for w in (L.VCT_WARP_NONE, L.VCT_WARP_PERSPECTIVE)],
                ids=lambda p: f"{p[0]}-{'persp' if p[1] else 'linear'}")
def tess(request):
    import torch

    name, mode = request.param
    sc = CASES[name]()
    g = GpuScene(sc)
    w = O.warp(sc, mode) if mode else None
    ref = O.voxelize_tess(sc, nthreads=8, warp=w)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc, voxelize_tesselation=1, warp_mode=mode))
    ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, sc.eye)
    torch.cuda.synchronize()
    got = split_records(*ctx.read_accumulators())
    ctx.normalize()
    torch.cuda.synchronize()
    return name, mode, sc, ref, got, ctx.stats()


def test_tess_accumulators_bitexact(tess):
    name, mode, sc, (count, sums, total), (gc, gs, gocc, pad), stats = tess
    assert count.sum() > 1000
    assert np.array_equal(gc, count)
    assert np.array_equal(gs, sums)
    assert np.array_equal(gocc, count > 0)
    assert np.all(pad == 0)
    assert stats["total_voxel_fragments"] == total
    assert stats["unique_voxels"] == int((count > 0).sum())
    assert stats["max_fragments_per_voxel"] == int(count.max())
    print(f"{name}: {total} points, {int((count > 0).sum())} voxels, max {int(count.max())} per voxel")


def test_tess_differs_from_rasterising(tess):
    name, mode, sc, (count, _, _), _, _ = tess
    if mode:
        pytest.skip("compared unwarped")
    raster, _, _ = O.voxelize(sc, O.render_shadowmap(sc), nthreads=8)
    assert not np.array_equal(raster > 0, count > 0)
    # the same surfaces: most occupied voxels agree
    both = np.logical_and(raster > 0, count > 0).sum()
    assert both > 0.5 * (count > 0).sum()


def test_slivers_exercise_the_aggregated_stores():
    """Columns of thin triangles put several points of one warp into one
    voxel; the summed stores equal one store per point (the oracle)."""
    import torch

    sc = scenes.large_family(seed=5, dim=64, shadow=512, gbuffer=(64, 36), n_boxes=4, n_cyl=6, cyl_segments=1024)
    g = GpuScene(sc)
    count, sums, total = O.voxelize_tess(sc, nthreads=8)
    assert count.max() >= 32
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc, voxelize_tesselation=1))
    ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, sc.eye)
    torch.cuda.synchronize()
    gc, gs, _, _ = split_records(*ctx.read_accumulators())
    assert np.array_equal(gc, count) and np.array_equal(gs, sums)


def _tess_volumes(sc, mode=L.VCT_WARP_NONE):
    """GPU tessellation voxelisation + normalisation: (records, colour, normal, stats)."""
    import torch

    g = GpuScene(sc)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc, voxelize_tesselation=1, warp_mode=mode))
    ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, sc.eye)
    torch.cuda.synchronize()
    rec = split_records(*ctx.read_accumulators())
    ctx.normalize()
    torch.cuda.synchronize()
    vols = [ctx.read_volume(v, 0).cpu().numpy().view(np.uint16) for v in (L.VCT_VOLUME_COLOR, L.VCT_VOLUME_NORMAL)]
    return rec, vols[0], vols[1], ctx.stats()


def _check_exact_past_the_packed_bound(sc, ref, got):
    count, sums, total = ref
    (gc, gs, gocc, _), color, normal, stats = got
    assert count.max() > 65537 and sums.max() >= 2 ** 32  # the case the packed record cannot sum alone
    # records the carry pass rewrote have bit 31 of the count set and their sums' float values
    rewritten = (gc >> 31) != 0
    assert rewritten.any() and np.all(count[rewritten] >= 65537)
    assert np.array_equal(gc & 0x7FFFFFFF, count) and np.array_equal(gocc, count > 0)
    small = np.tile(~rewritten, 6)  # elsewhere the record's halves are the sums themselves
    assert np.array_equal(gs[small], sums[small])
    big = np.tile(rewritten, 6)
    assert np.array_equal(gs[big].view(np.float32), sums[big].astype(np.float32))
    rcol, rnrm, _, rst = O.normalize(sc, count, sums, nthreads=8)
    assert np.array_equal(color, rcol) and np.array_equal(normal, rnrm)
    assert stats["error_flags"] == 0
    assert stats["total_voxel_fragments"] == total and stats["max_fragments_per_voxel"] == int(count.max())


def test_tess_sums_exact_past_65536_points_per_voxel():
    """1,600 coincident slivers put up to 185,600 points into one voxel and
    sums past 2^32 into its fields: the carry table keeps colour and normal
    bit-exact against the oracle's 64-bit sums, with no overflow flag."""
    sc = scenes.stacked_slivers(1600)
    _check_exact_past_the_packed_bound(sc, O.voxelize_tess(sc, nthreads=8), _tess_volumes(sc))


def test_large_frame_perspective_tess_exact():
    """The large frame through the tessellation voxeliser with the
    perspective warp (the reference's default voxeliser): up to ~91,000
    points fall into one froxel; colour and normal stay bit-exact."""
    sc = scenes.large(seed=0)
    w = O.warp(sc, L.VCT_WARP_PERSPECTIVE)
    _check_exact_past_the_packed_bound(sc, O.voxelize_tess(sc, nthreads=16, warp=w),
                                       _tess_volumes(sc, L.VCT_WARP_PERSPECTIVE))


@pytest.fixture(scope="module", params=[True, False], ids=["tess", "raster"])
def persp_frame(request):
    import torch

    tesselation = request.param
    sc = scenes.cornell(seed=7, gbuffer=(320, 180))
    g = GpuScene(sc)
    sm, gbuf = g.host_inputs()
    ref = O.frame(sc, shadowmap=sm, gbuf=gbuf, warp_mode=L.VCT_WARP_PERSPECTIVE, tesselation=tesselation,
                  nthreads=8)
    ref64 = O.trace(sc, ref["chain"], *gbuf, precision=64, want=("irr",), warp=ref["warp"], nthreads=8)
    prm = api.scene_params(sc, warp_mode=L.VCT_WARP_PERSPECTIVE, voxelize_tesselation=int(tesselation))
    # stage by stage
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(prm)
    ctx.voxelize(g.tris, g.lights, g.shadow, sc.eye)
    ctx.inject(g.shadow, sc.eye)
    ctx.build_mips()
    irr, spec, col, samples = g.new_outputs()
    ctx.trace(g.gb, sc.eye, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    stage = dict(chain=read_chain(ctx), irr=irr.cpu().numpy())
    # fused
    ctx2 = api.Context(api.config_for(sc))
    ctx2.set_params(prm)
    irr2, spec2, col2, samples2 = g.new_outputs()
    ctx2.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr2, spec2, col2, samples2))
    torch.cuda.synchronize()
    fused = dict(chain=read_chain(ctx2), irr=irr2.cpu().numpy(), stats=ctx2.stats())
    return tesselation, sc, ref, ref64, stage, fused


def test_perspective_frame_chain_bitexact(persp_frame):
    tesselation, sc, ref, _, stage, fused = persp_frame
    assert np.count_nonzero(ref["chain"]) > 1000
    assert np.array_equal(stage["chain"], ref["chain"])
    assert np.array_equal(fused["chain"], ref["chain"])
    assert fused["stats"]["total_voxel_fragments"] == ref["stats"]["total_voxel_fragments"]
    lin = O.frame(sc, shadowmap=ref["shadowmap"], gbuf=(ref["gpos"], ref["gnrm"], ref["galb"]),
                  tesselation=tesselation, nthreads=8, rows=(0, 1))
    if tesselation:  # the froxel grid differs from the linear one
        assert not np.array_equal(lin["count"] > 0, ref["count"] > 0)
    else:  # voxelize.frag ignores voxelizeTesselationWarp; injection and the trace do not
        assert np.array_equal(lin["count"], ref["count"])
        assert not np.array_equal(lin["chain"], ref["chain"])


def test_perspective_frame_trace(persp_frame):
    tesselation, sc, ref, ref64, stage, fused = persp_frame
    irr = rgb(stage["irr"])
    assert np.abs(irr).sum() > 0
    assert rel_l2(irr, rgb(ref["irradiance"])) <= 1e-5
    e64 = rel_l2(irr, rgb(ref64[0]))
    print(f"perspective warp ({'tess' if tesselation else 'raster'}): irradiance rel L2 vs fp64 {e64:.2e}")
    assert e64 <= 1e-3
    assert np.array_equal(stage["irr"].view(np.uint32), fused["irr"].view(np.uint32))


@pytest.mark.parametrize("mode", [L.VCT_WARP_NONE, L.VCT_WARP_PERSPECTIVE], ids=["linear", "persp"])
def test_batch_tesselation_equals_single_frames(mode):
    import torch

    scs = [scenes.batch_scene(seed=11, index=i) for i in range(3)]
    gs = [GpuScene(sc) for sc in scs]
    ref = []
    for sc, g in zip(scs, gs):
        ctx = api.Context(api.config_for(sc))
        ctx.set_params(api.scene_params(sc, voxelize_tesselation=1, warp_mode=mode))
        o = g.new_outputs()
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
        torch.cuda.synchronize()
        ref.append((read_chain(ctx), o[0].cpu().numpy(), ctx.stats()))
    b = api.Batch([api.config_for(sc) for sc in scs])
    for i, sc in enumerate(scs):
        b.set_params(api.scene_params(sc, voxelize_tesselation=1, warp_mode=mode), i)
    outs = [g.new_outputs() for g in gs]
    b.frame([api.scene_desc(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
             for sc, g, o in zip(scs, gs, outs)])
    torch.cuda.synchronize()
    for (chain, irr, st), ctx, o in zip(ref, b.scenes, outs):
        assert np.array_equal(read_chain(ctx), chain)
        assert np.array_equal(o[0].cpu().numpy().view(np.uint32), irr.view(np.uint32))
        assert ctx.stats()["total_voxel_fragments"] == st["total_voxel_fragments"] > 0


def test_batch_refuses_mixed_voxelisers():
    scs = [scenes.batch_scene(seed=1, index=i) for i in range(2)]
    gs = [GpuScene(sc) for sc in scs]
    b = api.Batch([api.config_for(sc) for sc in scs])
    b.set_params(api.scene_params(scs[0], voxelize_tesselation=1), 0)
    b.set_params(api.scene_params(scs[1]), 1)
    outs = [g.new_outputs() for g in gs]
    with pytest.raises(L.VctError) as e:
        b.frame([api.scene_desc(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
                 for sc, g, o in zip(scs, gs, outs)])
    assert e.value.status == L.VCT_ERR_INVALID_ARGUMENT


def test_batch_with_perspective_warp_equals_single_frames():
    import torch

    scs = [scenes.batch_scene(seed=7, index=i) for i in range(3)]
    gs = [GpuScene(sc) for sc in scs]
    ref = []
    for sc, g in zip(scs, gs):
        ctx = api.Context(api.config_for(sc))
        ctx.set_params(api.scene_params(sc, warp_mode=L.VCT_WARP_PERSPECTIVE))
        o = g.new_outputs()
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
        torch.cuda.synchronize()
        ref.append((read_chain(ctx), o[0].cpu().numpy()))
    b = api.Batch([api.config_for(sc) for sc in scs])
    for i, sc in enumerate(scs):
        b.set_params(api.scene_params(sc, warp_mode=L.VCT_WARP_PERSPECTIVE), i)
    outs = [g.new_outputs() for g in gs]
    b.frame([api.scene_desc(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
             for sc, g, o in zip(scs, gs, outs)])
    torch.cuda.synchronize()
    for (chain, irr), ctx, o in zip(ref, b.scenes, outs):
        assert np.array_equal(read_chain(ctx), chain)
        assert np.array_equal(o[0].cpu().numpy().view(np.uint32), irr.view(np.uint32))
