"""Parity scenes from OBJ meshes (the reference's resources/*.obj path):
generated OBJ texts loaded the way the reference's loader reads them, then
the whole frame with the rasterising voxeliser and the accumulators of the
tessellation voxeliser against the oracle."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from helpers import GpuScene, read_chain, rel_l2, rgb, split_records
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def obj_frame():
    import torch

    sph = scenes.icosphere(3) * 0.5 + np.array([-0.4, 0.0, 0.0])
    text = scenes.obj_text(sph, sph)
    sc = scenes.obj_scene(text, seed=3, dim=64, gbuffer=(320, 180))
    g = GpuScene(sc)
    sm, gbuf = g.host_inputs()
    ref = O.frame(sc, shadowmap=sm, gbuf=gbuf, nthreads=8)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc))
    irr, spec, col, samples = g.new_outputs()
    ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    return sc, g, ref, read_chain(ctx), irr.cpu().numpy(), ctx.stats()


def test_obj_frame_bitexact_volumes(obj_frame):
    sc, g, ref, chain, irr, stats = obj_frame
    assert np.count_nonzero(ref["chain"]) > 1000
    assert np.array_equal(chain, ref["chain"])
    assert stats["total_voxel_fragments"] == ref["stats"]["total_voxel_fragments"]


def test_obj_frame_trace(obj_frame):
    sc, g, ref, chain, irr, stats = obj_frame
    assert rel_l2(rgb(irr), rgb(ref["irradiance"])) <= 1e-5


def test_obj_quads_without_normals_tessellated():
    """Quads without normals (zero normals, as the reference's loader leaves
    them) through the tessellation voxeliser: normalize(0) is NaN in fp32, and
    the stored normal of those points is quantised the same way on both
    sides."""
    import torch

    box, _ = scenes._box(np.random.default_rng(1), np.array([0.9, 0.7, 0.8]), np.array([0.0, 0.0, 0.0]), 0.4)
    sc = scenes.obj_scene(scenes.obj_text(box, quads=True), seed=4, dim=64, gbuffer=(64, 36), walls=False)
    assert np.all(sc.normals == 0)
    g = GpuScene(sc)
    count, sums, total = O.voxelize_tess(sc, nthreads=8)
    assert count.sum() > 1000
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc, voxelize_tesselation=1))
    ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, sc.eye)
    torch.cuda.synchronize()
    gc, gs, _, _ = split_records(*ctx.read_accumulators())
    assert np.array_equal(gc, count) and np.array_equal(gs, sums)
