"""Dynamic scenes: rigid actors moved by vct_transform_actors (voxelize.vert's
model and normal matrices), re-voxelised every frame with the temporal
filter on (transferVoxels.comp:55-62 and the relit-voxel mix of
injectRadiance.comp:86-93), and the temporalRadianceFilter.comp decay; every
frame's radiance chain bit-exact against the oracle."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from helpers import read_chain, u16
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dyn():
    sc, actors = scenes.dynamic_scene(seed=2, n_actors=6, dim=64, shadow=512, gbuffer=(160, 90), static_boxes=200,
                                      static_cyl=4)
    return sc, actors


def test_transform_actors_bitexact(dyn):
    import torch

    sc, actors = dyn
    pos = torch.from_numpy(sc.positions).cuda()
    nrm = torch.from_numpy(sc.normals).cuda()
    alb = torch.from_numpy(sc.albedo).cuda()
    local = api.triangles(pos, nrm, alb)
    out_p, out_n = pos.clone(), nrm.clone()
    models = actors.models(0.7)
    api.transform_actors(local, models, out_p, out_n)
    torch.cuda.synchronize()
    rp, rn = O.transform_actors(sc.positions, sc.normals, actors.first, actors.count,
                                np.stack([m.T.reshape(16) for _, _, m in models]))
    assert np.array_equal(out_p.cpu().numpy().view(np.uint32), rp.view(np.uint32))
    assert np.array_equal(out_n.cpu().numpy().view(np.uint32), rn.view(np.uint32))
    # the static part is untouched, the actors moved
    s = int(actors.first[0])
    assert np.array_equal(rp[:s], sc.positions[:s]) and not np.array_equal(rp[s:], sc.positions[s:])


def test_rejects_overlapping_actor_ranges(dyn):
    import torch

    sc, actors = dyn
    pos = torch.from_numpy(sc.positions).cuda()
    local = api.triangles(pos, pos, torch.from_numpy(sc.albedo).cuda())
    bad = [(10, 100, np.eye(4)), (50, 10, np.eye(4))]
    with pytest.raises(L.VctError):
        api.transform_actors(local, bad, pos.clone(), pos.clone())


def test_temporal_frames_bitexact(dyn):
    import torch

    sc, actors = dyn
    N = sc.dim
    nv = N ** 3
    decay = 0.8
    pos0 = torch.from_numpy(sc.positions).cuda()
    nrm0 = torch.from_numpy(sc.normals).cuda()
    alb = torch.from_numpy(sc.albedo).cuda()
    local = api.triangles(pos0, nrm0, alb)
    pos, nrm = pos0.clone(), nrm0.clone()
    world = api.triangles(pos, nrm, alb)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc, temporal_filter=1, temporal_decay=decay, radiance_lighting=1))
    W, H = sc.gbuffer_size
    SW, SH = sc.shadow_size
    sm = torch.empty(SW * SH, device="cuda")
    keys = torch.empty(W * H, dtype=torch.int64, device="cuda")
    gpos, gnrm, galb = (torch.empty(W * H * 4, device="cuda") for _ in range(3))
    out = torch.empty(W * H * 4, device="cuda")
    chain = np.zeros(4 * O.chain_voxels(N, sc.levels), np.uint16)
    for f, t in enumerate((0.0, 0.25, 0.5)):
        models = actors.models(t)
        api.transform_actors(local, models, pos, nrm)
        api.render_shadowmap(world, sc, sm)
        api.render_gbuffer(world, sc, keys, gpos, gnrm, galb)
        ctx.frame(world, api.light_array(sc.lights), api.shadow_desc(sc, sm), sc.eye,
                  api.gbuffer(gpos, gnrm, galb, W, H), api.trace_out(color=out))
        torch.cuda.synchronize()
        got = read_chain(ctx)
        # oracle: the same frame through the stage functions, radiance carried over
        rp, rn = O.transform_actors(sc.positions, sc.normals, actors.first, actors.count,
                                    np.stack([m.T.reshape(16) for _, _, m in models]))
        smh = sm.cpu().numpy()
        count, sums, _ = O.voxelize(sc, smh, nthreads=8, positions=rp, normals=rn)
        color, normal, _, _ = O.normalize(sc, count, sums, temporal=1, decay=decay, radiance=chain, nthreads=8)
        O.inject(sc, smh, color, normal, chain, lighting=1, nthreads=8, temporal=1, decay=decay)
        O.build_mips(N, sc.levels, chain, 8)
        assert np.array_equal(got, chain), f"frame {f}"
    # the history matters: a frame from a fresh context differs
    fresh = api.Context(api.config_for(sc))
    fresh.set_params(api.scene_params(sc, temporal_filter=1, temporal_decay=decay, radiance_lighting=1))
    fresh.frame(world, api.light_array(sc.lights), api.shadow_desc(sc, sm), sc.eye,
                api.gbuffer(gpos, gnrm, galb, W, H), api.trace_out(color=out))
    torch.cuda.synchronize()
    assert not np.array_equal(read_chain(fresh), chain)
    # temporalRadianceFilter.comp
    ctx.decay_radiance()
    torch.cuda.synchronize()
    lvl0 = u16(ctx.read_volume(L.VCT_VOLUME_RADIANCE, 0))
    want = O.decay_radiance(chain[:4 * nv].copy(), decay)
    assert np.array_equal(lvl0, want)


def test_stage_inject_temporal_equals_fused():
    """vct_inject with the temporal filter and radianceLighting (marked voxels
    relit once from the seeded radiance) equals the fused frame."""
    import torch

    from helpers import GpuScene

    sc = scenes.cornell(seed=8)
    g = GpuScene(sc)
    p = api.scene_params(sc, temporal_filter=1, temporal_decay=0.7, radiance_lighting=1)
    a, b = api.Context(api.config_for(sc)), api.Context(api.config_for(sc))
    a.set_params(p)
    b.set_params(p)
    outs = g.new_outputs()
    for _ in range(2):
        a.voxelize(g.tris, g.lights, g.shadow, sc.eye)
        a.inject(g.shadow, sc.eye)
        a.build_mips()
        b.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(*outs))
        torch.cuda.synchronize()
        assert np.array_equal(read_chain(a), read_chain(b))


@pytest.mark.slow
def test_turned_slivers_accumulators_bitexact():
    """The full dynamic scene at 256^3 with its actors turned (t = 1 s): thin
    slivers whose bounding boxes hold about 15 times their covered pixels,
    rasterised in work units of whole rows narrowed to each row's span of the
    triangle.  The integer accumulators equal the oracle's, bit for bit."""
    import dataclasses
    import os

    import torch

    from helpers import GpuScene, split_records

    sc, actors = scenes.dynamic_scene(seed=0)
    models = actors.models(1.0)
    rp, rn = O.transform_actors(sc.positions, sc.normals, actors.first, actors.count,
                                np.stack([m.T.reshape(16) for _, _, m in models]))
    moved = dataclasses.replace(sc, positions=np.ascontiguousarray(rp, np.float32).reshape(sc.positions.shape),
                                normals=np.ascontiguousarray(rn, np.float32).reshape(sc.normals.shape))
    g = GpuScene(moved)
    torch.cuda.synchronize()
    count, sums, total = O.voxelize(moved, g.sm.cpu().numpy(), nthreads=os.cpu_count() or 1)
    with api.Context(api.config_for(moved)) as ctx:
        ctx.set_params(api.scene_params(moved))
        ctx.voxelize_accumulate(g.tris, g.lights, g.shadow, moved.eye)
        torch.cuda.synchronize()
        c, s, occ, _ = split_records(*ctx.read_accumulators())
        assert ctx.stats()["total_voxel_fragments"] == total
    assert np.array_equal(c, count)
    assert np.array_equal(s, sums)
    assert np.array_equal(occ, count > 0)
