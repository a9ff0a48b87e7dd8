"""Launch-shape tuning: every voxeliser work-unit size, raster occupancy and
trace tile / warp shape gives bit-identical volumes and trace outputs, and
the autotuner returns a valid setting for a context and for a batch."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import GpuScene, read_chain
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu

TILES = [(16, 16, 8), (16, 16, 4), (16, 16, 16), (32, 8, 8), (32, 8, 4), (32, 8, 16), (32, 8, 32), (8, 32, 4),
         (8, 32, 8), (64, 4, 8), (64, 4, 16), (64, 4, 32), (4, 64, 4)]


@pytest.fixture(scope="module")
def scene():
    # 640x360 does not divide into 64x4 or 4x64 tiles: partial tiles are covered.
    sc = scenes.cornell(seed=5, gbuffer=(636, 358))
    return sc, GpuScene(sc)


def _run(ctx, sc, g):
    import torch

    irr, spec, col, samples = g.new_outputs()
    ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    return dict(chain=read_chain(ctx), irr=irr.cpu().numpy(), spec=spec.cpu().numpy(), col=col.cpu().numpy(),
                samples=int(samples.item()), stats=ctx.stats())


def _same(a, b, what):
    assert a["stats"] == b["stats"], what
    assert a["samples"] == b["samples"], what
    for k in ("chain", "irr", "spec", "col"):
        assert np.array_equal(a[k].view(np.uint32 if k != "chain" else np.uint16),
                              b[k].view(np.uint32 if k != "chain" else np.uint16)), f"{what}: {k}"


def test_every_launch_shape_gives_identical_results(scene):
    sc, g = scene
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc))
    ref = _run(ctx, sc, g)
    for unit in (32, 128, 512, 2048, 8192):
        for bps in (1, 2, 3):
            ctx.set_tuning(api.tuning_from(dict(voxel_unit_pixels=unit, voxel_blocks_per_sm=bps)))
            _same(_run(ctx, sc, g), ref, f"unit {unit} bps {bps}")
    for tw, th, ww in TILES:
        ctx.set_tuning(api.tuning_from(dict(trace_tile_w=tw, trace_tile_h=th, trace_warp_w=ww)))
        _same(_run(ctx, sc, g), ref, f"tile {tw}x{th} warp {ww}")
    ctx.close()


@pytest.mark.parametrize("bad", [dict(voxel_unit_pixels=100), dict(voxel_unit_pixels=16), dict(voxel_blocks_per_sm=4),
                                 dict(trace_tile_w=16, trace_tile_h=8), dict(trace_warp_w=32),
                                 dict(trace_tile_w=64, trace_tile_h=4, trace_warp_w=4)])
def test_invalid_tuning_rejected(scene, bad):
    sc, _ = scene
    ctx = api.Context(api.config_for(sc))
    before = api.tuning_dict(ctx.tuning())
    with pytest.raises(L.VctError):
        ctx.set_tuning(api.tuning_from(bad))
    assert api.tuning_dict(ctx.tuning()) == before
    ctx.close()


def test_autotune_context(scene):
    sc, g = scene
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc))
    ref = _run(ctx, sc, g)
    irr, spec, col, samples = g.new_outputs()
    best = ctx.autotune(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples), reps=2)
    t = api.tuning_dict(best)
    assert t == api.tuning_dict(ctx.tuning())
    assert t["voxel_unit_pixels"] in (128, 256, 512, 1024, 2048)
    assert t["trace_tile_w"] * t["trace_tile_h"] == 256
    _same(_run(ctx, sc, g), ref, "after autotune")
    ctx.close()


def test_autotune_batch():
    import torch

    scs = [scenes.batch_scene(seed=21, index=i) for i in range(4)]
    gs = [GpuScene(sc) for sc in scs]
    cfgs = [api.config_for(sc) for sc in scs]
    b = api.Batch(cfgs)
    for i, sc in enumerate(scs):
        b.set_params(api.scene_params(sc), i)
    outs = [g.new_outputs() for g in gs]
    descs = [api.scene_desc(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
             for sc, g, o in zip(scs, gs, outs)]
    b.frame(descs)
    torch.cuda.synchronize()
    ref = [o[0].clone() for o in outs]
    best = b.autotune(descs, reps=2)
    assert api.tuning_dict(best) == api.tuning_dict(b.tuning())
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    b.capture(descs, stream)
    for o in outs:
        o[0].zero_()
    stream.wait_stream(torch.cuda.current_stream())  # the zeroing runs on the default stream
    b.replay(stream)
    stream.synchronize()
    for o, r in zip(outs, ref):
        assert torch.equal(o[0].view(torch.int32), r.view(torch.int32))
    b.close()
