"""Edge cases of the frame against the oracle: no triangles, geometry
outside the volume, no lights, degenerate and viewport-filling triangles
(both voxelisers), shadow maps and G-buffers whose sizes are not multiples of
16 (injectRadiance's `>` bound), and a chain with fewer levels than the grid
allows.  Volumes bit-exact, irradiance within the trace tolerance."""

from __future__ import annotations

import dataclasses

import numpy as np
import pytest

import oracle as O
from helpers import GpuScene, read_chain, rel_l2, rgb
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _with(sc, tris, nrms=None, alb=None, **kw):
    tris = np.asarray(tris, dtype=np.float32).reshape(-1, 9)
    if nrms is None:
        t = tris.reshape(-1, 3, 3).astype(np.float64)
        n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
        ln = np.linalg.norm(n, axis=1, keepdims=True)
        n = np.where(ln > 0, n / np.maximum(ln, 1e-30), np.array([0.0, 1.0, 0.0]))
        nrms = np.repeat(n[:, None, :], 3, axis=1)
    if alb is None:
        alb = np.random.default_rng(len(tris)).uniform(0.1, 0.9, size=(len(tris), 3))
    return dataclasses.replace(sc, positions=np.ascontiguousarray(tris, dtype=np.float32),
                               normals=np.ascontiguousarray(np.asarray(nrms).reshape(-1, 9), dtype=np.float32),
                               albedo=np.ascontiguousarray(alb, dtype=np.float32), **kw)


def _run(sc, levels=None, tess=False):
    import torch

    g = GpuScene(sc)
    sm, gbuf = g.host_inputs()
    ref = O.frame(sc, shadowmap=sm, gbuf=gbuf, nthreads=8, tesselation=tess)
    cfg = api.config_for(sc)
    if levels:
        cfg.voxel_levels = levels
    ctx = api.Context(cfg)
    ctx.set_params(api.scene_params(sc, voxelize_tesselation=int(tess)))
    irr, spec, col, samples = g.new_outputs()
    ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    return ref, read_chain(ctx), irr.cpu().numpy(), ctx.stats()


def _check(ref, chain, irr, stats):
    assert np.array_equal(chain, ref["chain"])
    assert stats["total_voxel_fragments"] == ref["stats"]["total_voxel_fragments"]
    assert stats["unique_voxels"] == ref["stats"]["unique_voxels"]
    assert stats["max_fragments_per_voxel"] == ref["stats"]["max_fragments_per_voxel"]
    r = rgb(ref["irradiance"])
    if np.abs(r).sum() == 0:
        assert np.abs(rgb(irr)).sum() == 0
    else:
        assert rel_l2(rgb(irr), r) <= 1e-5


def test_no_triangles():
    sc = _with(scenes.cornell(seed=1, gbuffer=(64, 36)), np.zeros((0, 9)))
    ref, chain, irr, stats = _run(sc)
    _check(ref, chain, irr, stats)
    assert not chain.any() and stats["total_voxel_fragments"] == 0 and stats["unique_voxels"] == 0


def test_geometry_outside_the_volume():
    base = scenes.cornell(seed=2, gbuffer=(96, 54))
    t = base.positions.reshape(-1, 3, 3) + np.array([3.0, 0.0, 0.0], np.float32)
    sc = _with(base, t, base.normals, base.albedo)
    ref, chain, irr, stats = _run(sc)
    _check(ref, chain, irr, stats)
    assert stats["unique_voxels"] == 0


@pytest.mark.parametrize("tess", [False, True], ids=["raster", "tess"])
def test_no_lights(tess):
    sc = dataclasses.replace(scenes.cornell(seed=3, gbuffer=(96, 54)), lights=[])
    ref, chain, irr, stats = _run(sc, tess=tess)
    _check(ref, chain, irr, stats)
    assert stats["unique_voxels"] > 0


@pytest.mark.parametrize("tess", [False, True], ids=["raster", "tess"])
def test_degenerate_and_viewport_filling_triangles(tess):
    base = scenes.cornell(seed=4, gbuffer=(96, 54))
    p = np.array([0.1, 0.2, 0.3])
    degenerate = [
        np.concatenate([p, p, p]),                                            # a point
        np.concatenate([p, p + [0.3, 0.0, 0.0], p + [0.6, 0.0, 0.0]]),        # collinear
        np.concatenate([p, p, p + [0.0, 0.5, 0.0]]),                          # repeated vertex
    ]
    big = [np.array([-3.0, -3.0, 0.05, 3.0, -3.0, 0.05, 0.0, 3.0, 0.05])]  # beyond every side of the volume
    tris = np.concatenate([base.positions, np.array(degenerate), np.array(big)])
    sc = _with(base, tris)
    ref, chain, irr, stats = _run(sc, tess=tess)
    _check(ref, chain, irr, stats)
    assert stats["unique_voxels"] > 0


def test_ragged_sizes_and_fewer_levels():
    # a 100 x 60 shadow map (the inject dispatch runs index == size), a 97 x 53 G-buffer,
    # a 32^3 grid with 3 levels instead of 6
    sc = scenes.cornell(seed=5, dim=32, shadow=100, gbuffer=(97, 53))
    sc = dataclasses.replace(sc, shadow_size=(100, 60), levels=3)
    ref, chain, irr, stats = _run(sc, levels=3)
    _check(ref, chain, irr, stats)
    assert len(chain) == 4 * sum((32 >> l) ** 3 for l in range(3))
