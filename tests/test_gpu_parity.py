"""Parity of every stage of the CUDA path (through the C ABI) with the CPU
oracle on the same seeded inputs.

Bars:
  - shadow map, accumulators, occupancy, colour/normal/radiance volumes,
    mip chain, VoxelizeInfo counters: bit-exact;
  - irradiance (software sampler): relative L2 error <= 1e-5 against the fp32
    oracle and <= 1e-3 against the fp64 oracle; 99.9% of pixels within 1e-3
    relative (a pixel may flip one early-out step on a rounding tie);
  - irradiance (texture-unit sampler): relative L2 error <= 1e-2 against fp64
    (its filter weights are 8-bit fixed point), reported.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from helpers import GpuScene, read_chain, rel_l2, rgb, split_records, u16, u32
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cornell():
    sc = scenes.cornell(seed=0)
    g = GpuScene(sc)
    sm, gbuf = g.host_inputs()
    ref = O.frame(sc, shadowmap=sm, gbuf=gbuf)
    ref64 = O.trace(sc, ref["chain"], *gbuf, precision=64, want=("irr", "spec"))
    return sc, g, ref, ref64


def run_stages(sc, g, params=None, hardware=False):
    import torch

    ctx = api.Context(api.config_for(sc))
    p = params or api.scene_params(sc)
    if hardware:
        p.trace_filter = L.VCT_FILTER_HARDWARE
    ctx.set_params(p)
    ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, sc.eye)
    torch.cuda.synchronize()
    cnt, sums, occ, pad = split_records(*ctx.read_accumulators())
    ctx.normalize()
    torch.cuda.synchronize()
    after = split_records(*ctx.read_accumulators())
    color0 = u16(ctx.read_volume(L.VCT_VOLUME_COLOR, 0))
    normal0 = u16(ctx.read_volume(L.VCT_VOLUME_NORMAL, 0))
    rad_seed = u16(ctx.read_volume(L.VCT_VOLUME_RADIANCE, 0))
    ctx.inject(g.shadow, sc.eye)
    ctx.build_mips()
    irr, spec, col, samples = g.new_outputs()
    ctx.trace(g.gb, sc.eye, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    out = dict(count=cnt, sums=sums, occ=occ, pad=pad, after=after, color=color0, normal=normal0, rad_seed=rad_seed, chain=read_chain(ctx),
               irr=irr.cpu().numpy(), spec=spec.cpu().numpy(), col=col.cpu().numpy(),
               samples=int(samples.item()), stats=ctx.stats())
    ctx.close()
    return out


def test_shadowmap_bitexact(cornell):
    sc, g, ref, _ = cornell
    assert np.array_equal(g.sm.cpu().numpy().view(np.uint32), O.render_shadowmap(sc).view(np.uint32))


def test_gbuffer_matches_oracle(cornell):
    sc, g, _, _ = cornell
    gp, gn, ga = O.render_gbuffer(sc)
    a = g.gpos.cpu().numpy().reshape(-1, 4)
    b = gp.reshape(-1, 4)
    assert np.array_equal(a[:, 3], b[:, 3])
    assert np.array_equal(a, b)
    assert np.array_equal(g.gnrm.cpu().numpy(), gn)
    assert np.array_equal(g.galb.cpu().numpy(), ga)


@pytest.fixture(scope="module")
def stages(cornell):
    sc, g, _, _ = cornell
    return run_stages(sc, g)


def test_accumulators_bitexact(cornell, stages):
    sc, g, ref, _ = cornell
    assert np.array_equal(stages["count"], ref["count"])
    assert np.array_equal(stages["sums"], ref["sums"])
    assert (stages["count"] > 0).sum() == ref["stats"]["unique_voxels"]
    # occupancy mask is exactly the set of voxels with fragments
    assert np.array_equal(stages["occ"], ref["count"] > 0)
    assert not stages["pad"].any()


def test_normalize_leaves_accumulators_zero(stages):
    count, sums, occ, pad = stages["after"]
    assert not count.any() and not sums.any() and not occ.any() and not pad.any()


def test_normalize_bitexact(cornell, stages):
    sc, g, ref, _ = cornell
    assert np.array_equal(stages["color"], ref["color"])
    assert np.array_equal(stages["normal"], ref["normal"])


def test_stats_match(cornell, stages):
    _, _, ref, _ = cornell
    st = stages["stats"]
    for k in ("total_voxel_fragments", "unique_voxels", "max_fragments_per_voxel", "error_flags"):
        assert st[k] == ref["stats"][k], k


def test_inject_and_mips_bitexact(cornell, stages):
    _, _, ref, _ = cornell
    assert np.array_equal(stages["chain"], ref["chain"])


def test_trace_software_matches_oracles(cornell, stages):
    sc, g, ref, ref64 = cornell
    irr = rgb(stages["irr"])
    assert rel_l2(irr, rgb(ref["irradiance"])) <= 1e-5
    e64 = rel_l2(irr, rgb(ref64[0]))
    assert e64 <= 1e-3, e64
    b = rgb(ref64[0]).astype(np.float64)
    per_px = np.abs(irr - b).max(1) / np.maximum(np.abs(b).max(1), 1e-3)
    assert np.quantile(per_px, 0.999) <= 1e-3
    assert rel_l2(rgb(stages["spec"]), rgb(ref64[1])) <= 1e-3
    assert stages["samples"] == pytest.approx(ref["samples"], rel=1e-3)


def test_composite_color(cornell, stages):
    _, _, ref, _ = cornell
    assert rel_l2(rgb(stages["col"]), rgb(ref["out"])) <= 1e-4


def test_trace_hardware_sampler(cornell):
    sc, g, ref, ref64 = cornell
    hw = run_stages(sc, g, hardware=True)
    assert np.array_equal(hw["chain"], ref["chain"])
    e = rel_l2(rgb(hw["irr"]), rgb(ref64[0]))
    print(f"hardware sampler irradiance rel-L2 vs fp64: {e:.3e}")
    assert e <= 1e-2


def test_frame_fused_hardware_sampler(cornell):
    """The fused frame writes the texture-unit copy of the mip chain through
    surfaces; tracing it must give exactly what the staged path (which copies
    the linear chain into the array) gives."""
    import torch

    sc, g, ref, ref64 = cornell
    staged = run_stages(sc, g, hardware=True)
    with api.Context(api.config_for(sc)) as ctx:
        ctx.set_params(api.scene_params(sc, trace_filter=L.VCT_FILTER_HARDWARE))
        irr, spec, col, samples = g.new_outputs()
        for _ in range(2):
            ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
        torch.cuda.synchronize()
        assert np.array_equal(read_chain(ctx), ref["chain"])
        assert np.array_equal(irr.cpu().numpy(), staged["irr"])
        assert np.array_equal(spec.cpu().numpy(), staged["spec"])


def test_frame_fused_equals_stages(cornell, stages):
    import torch

    sc, g, ref, _ = cornell
    with api.Context(api.config_for(sc)) as ctx:
        ctx.set_params(api.scene_params(sc))
        irr, spec, col, samples = g.new_outputs()
        for _ in range(2):  # second frame checks that the accumulators/lit mask were cleared
            ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
        torch.cuda.synchronize()
        assert np.array_equal(read_chain(ctx), ref["chain"])
        assert np.array_equal(u16(ctx.read_volume(L.VCT_VOLUME_COLOR, 0)), ref["color"])
        assert np.array_equal(irr.cpu().numpy(), stages["irr"])
        assert np.array_equal(col.cpu().numpy(), stages["col"])
        st = ctx.stats()
        assert st["unique_voxels"] == ref["stats"]["unique_voxels"]
        assert st["total_voxel_fragments"] == ref["stats"]["total_voxel_fragments"]


def test_triangle_order_independence(cornell, stages):
    import torch

    sc, _, _, _ = cornell
    perm = np.random.default_rng(7).permutation(sc.ntri)
    sc2 = scenes.cornell(seed=0)
    sc2.positions = np.ascontiguousarray(sc.positions[perm])
    sc2.normals = np.ascontiguousarray(sc.normals[perm])
    sc2.albedo = np.ascontiguousarray(sc.albedo[perm])
    g2 = GpuScene(sc2)
    with api.Context(api.config_for(sc2)) as ctx:
        ctx.set_params(api.scene_params(sc2))
        ctx.voxelize_accumulate(g2.tris, g2.lights, g2.shadow, sc2.eye)
        torch.cuda.synchronize()
        cnt, sums, _, _ = split_records(*ctx.read_accumulators())
    assert np.array_equal(cnt, stages["count"])
    assert np.array_equal(sums, stages["sums"])


@pytest.mark.parametrize("opt", [dict(radiance_lighting=1), dict(radiance_dilate=1), dict(voxelize_lighting=0),
                                 dict(axis_override=1), dict(voxel_set_opacity=0.0)])
def test_options_bitexact(opt):
    import torch

    sc = scenes.tiny(seed=3)
    g = GpuScene(sc)
    sm, gbuf = g.host_inputs()
    with api.Context(api.config_for(sc)) as ctx:
        ctx.set_params(api.scene_params(sc, **opt))
        ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, sc.eye)
        torch.cuda.synchronize()
        cnt, sums, _, _ = split_records(*ctx.read_accumulators())
        ctx.normalize()
        ctx.inject(g.shadow, sc.eye)
        ctx.build_mips()
        torch.cuda.synchronize()
        chain = read_chain(ctx)
        # fused frame on a second context must agree too
    count, rsums, _ = O.voxelize(sc, sm, lighting=opt.get("voxelize_lighting", 1),
                                 axis_override=opt.get("axis_override", -1))
    assert np.array_equal(cnt, count)
    assert np.array_equal(sums, rsums)
    rchain = np.zeros(4 * O.chain_voxels(sc.dim, sc.levels), dtype=np.uint16)
    color, normal, _, _ = O.normalize(sc, count, rsums, opacity=opt.get("voxel_set_opacity", 0.5), radiance=rchain)
    O.inject(sc, sm, color, normal, rchain, lighting=opt.get("radiance_lighting", 0),
             dilate=opt.get("radiance_dilate", 0))
    O.build_mips(sc.dim, sc.levels, rchain)
    assert np.array_equal(chain, rchain)
    with api.Context(api.config_for(sc)) as ctx:
        ctx.set_params(api.scene_params(sc, **opt))
        irr, spec, col, samples = g.new_outputs()
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
        torch.cuda.synchronize()
        assert np.array_equal(read_chain(ctx), rchain)


def test_temporal_filter_bitexact():
    import torch

    sc = scenes.tiny(seed=4)
    g = GpuScene(sc)
    sm, _ = g.host_inputs()
    rchain = np.zeros(4 * O.chain_voxels(sc.dim, sc.levels), dtype=np.uint16)
    with api.Context(api.config_for(sc)) as ctx:
        ctx.set_params(api.scene_params(sc, temporal_filter=1, temporal_decay=0.8))
        for _ in range(3):
            ctx.voxelize(g.tris, g.lights, g.shadow, sc.eye)
            ctx.inject(g.shadow, sc.eye)
            ctx.build_mips()
            count, rsums, _ = O.voxelize(sc, sm)
            color, normal, _, _ = O.normalize(sc, count, rsums, temporal=1, decay=0.8, radiance=rchain)
            O.inject(sc, sm, color, normal, rchain)
            O.build_mips(sc.dim, sc.levels, rchain)
        torch.cuda.synchronize()
        assert np.array_equal(read_chain(ctx), rchain)


def test_hybrid_sampler_staged_and_fused(cornell):
    """VCT_FILTER_HYBRID: the finer level of each sample exact, the coarser
    by the texture units.  Held to the 1e-3 fp64 target; the fused frame
    (surfaces and bordered chain written by the resolve) equals the staged
    path (texture refreshed from the linear chain, bordered chain copied)."""
    import torch

    sc, g, ref, ref64 = cornell
    p = api.scene_params(sc, trace_filter=L.VCT_FILTER_HYBRID)
    staged = run_stages(sc, g, params=p)
    assert np.array_equal(staged["chain"], ref["chain"])
    e = rel_l2(rgb(staged["irr"]), rgb(ref64[0]))
    print(f"hybrid sampler irradiance rel-L2 vs fp64: {e:.3e}")
    assert e <= 1e-3
    with api.Context(api.config_for(sc)) as ctx:
        ctx.set_params(api.scene_params(sc, trace_filter=L.VCT_FILTER_HYBRID))
        irr, spec, col, samples = g.new_outputs()
        for _ in range(2):
            ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
        torch.cuda.synchronize()
        assert np.array_equal(irr.cpu().numpy(), staged["irr"])
        assert np.array_equal(spec.cpu().numpy(), staged["spec"])
        # levels 0-3 of the linear chain come back from the texture array
        assert np.array_equal(read_chain(ctx), ref["chain"])


def test_hybrid_frame_then_stage_paths(cornell):
    """A fused hybrid frame without the temporal filter leaves the linear copy
    of radiance levels 0-3 to the texture array.  The entry points that read
    the linear chain copy it back first: build_mips, a temporal frame (which
    reads last frame's level 0) and the radiance decay give the chain a
    software-sampler context, which writes every linear level, holds."""
    import torch

    sc, g, ref, _ = cornell
    chains = {}
    for filt in (L.VCT_FILTER_SOFTWARE, L.VCT_FILTER_HYBRID):
        with api.Context(api.config_for(sc)) as ctx:
            ctx.set_params(api.scene_params(sc, trace_filter=filt))
            irr, spec, col, samples = g.new_outputs()
            ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
            ctx.build_mips()
            torch.cuda.synchronize()
            assert np.array_equal(read_chain(ctx), ref["chain"])
            ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
            ctx.set_params(api.scene_params(sc, trace_filter=filt, temporal_filter=1, temporal_decay=0.8))
            ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
            ctx.decay_radiance()
            ctx.build_mips()
            torch.cuda.synchronize()
            chains[filt] = read_chain(ctx)
    assert np.array_equal(chains[L.VCT_FILTER_SOFTWARE], chains[L.VCT_FILTER_HYBRID])
    assert not np.array_equal(chains[L.VCT_FILTER_HYBRID], ref["chain"])
