"""Batched scenes: one launch per stage over scenes of uneven triangle
counts, grids and G-buffer sizes must give, scene by scene, exactly what
vct_frame gives for that scene alone (radiance chain, trace outputs and
VoxelizeInfo counters bit-exact), both run directly and replayed from the
captured CUDA graph."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import GpuScene, read_chain
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _configs_and_scenes():
    scs = [scenes.batch_scene(seed=11, index=i) for i in range(5)]
    cfgs = [api.config_for(sc) for sc in scs]
    # A grid whose chain is complete after the resolve (three levels).
    sc = scenes.cornell(seed=3, dim=64, gbuffer=(320, 180))
    c = api.config_for(sc)
    c.voxel_levels = 3
    scs.append(sc)
    cfgs.append(c)
    # An empty scene: no triangles, nothing voxelised, the trace still runs.
    sc = scenes.tiny(seed=2, dim=32, gbuffer=(64, 40))
    scs.append(sc)
    cfgs.append(api.config_for(sc))
    return scs, cfgs


@pytest.fixture(scope="module")
def setup():
    scs, cfgs = _configs_and_scenes()
    gs = [GpuScene(sc) for sc in scs]
    gs[-1].tris.count = 0
    return scs, cfgs, gs


def _outputs(g):
    return g.new_outputs()


def _read(ctx, outs):
    irr, spec, col, samples = outs
    return dict(chain=read_chain(ctx), irr=irr.cpu().numpy(), spec=spec.cpu().numpy(), col=col.cpu().numpy(),
                samples=int(samples.item()), stats=ctx.stats())


def _single(scs, cfgs, gs, filt):
    import torch

    res = []
    for sc, cfg, g in zip(scs, cfgs, gs):
        ctx = api.Context(cfg)
        ctx.set_params(api.scene_params(sc, trace_filter=filt))
        outs = _outputs(g)
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*outs))
        torch.cuda.synchronize()
        res.append(_read(ctx, outs))
        ctx.close()
    return res


def _descs(scs, gs, outs):
    return [api.scene_desc(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*o))
            for sc, g, o in zip(scs, gs, outs)]


def _same(a, b, what):
    assert a["stats"] == b["stats"], what
    assert a["samples"] == b["samples"], what
    for k in ("chain", "irr", "spec", "col"):
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), f"{what}: {k}"


@pytest.mark.parametrize("filt", [L.VCT_FILTER_SOFTWARE, L.VCT_FILTER_HARDWARE, L.VCT_FILTER_HYBRID])
def test_batch_frame_equals_single_frames(setup, filt):
    import torch

    scs, cfgs, gs = setup
    ref = _single(scs, cfgs, gs, filt)
    b = api.Batch(cfgs)
    for i, sc in enumerate(scs):
        b.set_params(api.scene_params(sc, trace_filter=filt), i)
    outs = [_outputs(g) for g in gs]
    descs = _descs(scs, gs, outs)
    # Two frames: the second must not see state left by the first.
    for _ in range(2):
        for o in outs:
            for t in o:
                t.zero_()
        b.frame(descs)
        torch.cuda.synchronize()
        for i in range(len(scs)):
            _same(_read(b.scenes[i], outs[i]), ref[i], f"scene {i}")
    b.close()


def test_batch_graph_replay_equals_single_frames(setup):
    import torch

    scs, cfgs, gs = setup
    ref = _single(scs, cfgs, gs, L.VCT_FILTER_SOFTWARE)
    b = api.Batch(cfgs)
    for i, sc in enumerate(scs):
        b.set_params(api.scene_params(sc), i)
    outs = [_outputs(g) for g in gs]
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    b.capture(_descs(scs, gs, outs), stream)
    for _ in range(3):
        with torch.cuda.stream(stream):
            for o in outs:
                for t in o:
                    t.zero_()
        b.replay(stream)
        stream.synchronize()
        for i in range(len(scs)):
            _same(_read(b.scenes[i], outs[i]), ref[i], f"replay scene {i}")
    b.close()


def test_batch_rejects_mixed_filters_and_wrong_count(setup):
    scs, cfgs, gs = setup
    b = api.Batch(cfgs[:2])
    b.set_params(api.scene_params(scs[0]), 0)
    b.set_params(api.scene_params(scs[1], trace_filter=L.VCT_FILTER_HARDWARE), 1)
    outs = [_outputs(g) for g in gs[:2]]
    with pytest.raises(L.VctError):
        b.frame(_descs(scs[:2], gs[:2], outs))
    b.set_params(api.scene_params(scs[1]), 1)
    with pytest.raises(L.VctError):
        b.frame(_descs(scs[:1], gs[:1], outs[:1]))
    with pytest.raises(L.VctError):
        b.replay()
    b.close()
