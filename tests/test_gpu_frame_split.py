"""vct_frame_volume + vct_trace (whole frame, or the frame traced in row
bands through G-buffer sub-views) equal vct_frame bit for bit, and the
stage timers cover the split frame."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import GpuScene, read_chain
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def test_split_frame_equals_frame():
    import torch

    sc = scenes.cornell(seed=8, gbuffer=(320, 180))
    g = GpuScene(sc)
    W, H = sc.gbuffer_size
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc))
    irr, spec, col, samples = g.new_outputs()
    ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    ref = [t.cpu().clone() for t in (irr, spec, col)]
    ref_chain = read_chain(ctx)

    ctx2 = api.Context(api.config_for(sc))
    ctx2.set_params(api.scene_params(sc))
    ctx2.enable_timers(True)
    irr2, spec2, col2, _ = g.new_outputs()
    ctx2.frame_volume(g.tris, g.lights, g.shadow, sc.eye)
    bands = [(0, 67), (67, 128), (128, H)]
    rows = lambda t, r0, r1: t[r0 * W * 4:r1 * W * 4]  # noqa: E731
    for r0, r1 in bands:
        gb = api.gbuffer(rows(g.gpos, r0, r1), rows(g.gnrm, r0, r1), rows(g.galb, r0, r1), W, r1 - r0)
        ctx2.trace(gb, sc.eye, api.trace_out(rows(irr2, r0, r1), rows(spec2, r0, r1), rows(col2, r0, r1)))
    torch.cuda.synchronize()
    assert np.array_equal(read_chain(ctx2), ref_chain)
    for a, b in zip(ref, (irr2, spec2, col2)):
        assert torch.equal(a.view(torch.int32), b.cpu().view(torch.int32))
    t = ctx2.timers()
    assert t["render_ms"] > 0 and t["total_ms"] >= t["render_ms"]


def test_frame_captured_in_a_cuda_graph():
    """vct_frame inside a caller's stream capture (its side-stream fork and
    join are events, which capture records): replays equal direct frames."""
    import torch

    sc = scenes.cornell(seed=10, gbuffer=(160, 90))
    g = GpuScene(sc)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc))
    irr, spec, col, samples = g.new_outputs()
    out = api.trace_out(irr, spec, col)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # the inputs were rendered on the default stream
    with torch.cuda.stream(s):
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, out, s)  # sizes the work arrays before capture
    s.synchronize()
    ref = irr.clone()
    chain_ref = read_chain(ctx)
    irr.zero_()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, out, s)
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(irr.view(torch.int32), ref.view(torch.int32))
    assert np.array_equal(read_chain(ctx), chain_ref)


def test_frames_in_flight_equal_frames():
    """The integration pattern with frames in flight: the next frame's
    uploads on a copy stream once this frame's volume pass has read its
    inputs, G-buffers double-buffered, images read back on a second copy
    stream during the next volume pass.  Two scenes alternate, so an upload
    that overtook a pass it must wait for would change an image."""
    import torch

    scs = [scenes.cornell(seed=s, gbuffer=(320, 180)) for s in (21, 22)]
    gs = [GpuScene(sc) for sc in scs]
    W, H = scs[0].gbuffer_size
    refs = []
    for sc, g in zip(scs, gs):
        ctx = api.Context(api.config_for(sc))
        ctx.set_params(api.scene_params(sc))
        irr, spec, col, _ = g.new_outputs()
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(color=col))
        torch.cuda.synchronize()
        refs.append(col.cpu().clone())
    assert not torch.equal(refs[0], refs[1])
    host = [[getattr(g, n).cpu().pin_memory() for n in ("pos", "nrm", "alb", "sm", "gpos", "gnrm", "galb")]
            for g in gs]
    d_in = [torch.empty_like(t, device="cuda:0") for t in host[0][:4]]
    d_gb = [[torch.empty_like(t, device="cuda:0") for t in host[0][4:]] for _ in range(2)]
    d_col = [torch.empty(W * H * 4, device="cuda:0") for _ in range(2)]
    tris = api.triangles(*d_in[:3])
    ctx = api.Context(api.config_for(scs[0]))
    ctx.set_params(api.scene_params(scs[0]))
    stream, up, down = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    ev_tri, ev_vol = torch.cuda.Event(), torch.cuda.Event()
    ev_gb, ev_done, ev_d2h = ([torch.cuda.Event(), torch.cuda.Event()] for _ in range(3))
    steps = 6
    out = [torch.empty(W * H * 4).pin_memory() for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        par, s = k & 1, k % 2
        up.wait_event(ev_vol)
        with torch.cuda.stream(up):
            for d, h in zip(d_in, host[s][:4]):
                d.copy_(h, non_blocking=True)
            ev_tri.record(up)
            up.wait_event(ev_done[par])
            for d, h in zip(d_gb[par], host[s][4:]):
                d.copy_(h, non_blocking=True)
            ev_gb[par].record(up)
        stream.wait_event(ev_tri)
        ctx.frame_volume(tris, gs[s].lights, api.shadow_desc(scs[s], d_in[3]), scs[s].eye, stream)
        ev_vol.record(stream)
        stream.wait_event(ev_gb[par])
        stream.wait_event(ev_d2h[par])
        ctx.trace(api.gbuffer(*d_gb[par], W, H), scs[s].eye, api.trace_out(color=d_col[par]), stream)
        ev_done[par].record(stream)
        with torch.cuda.stream(down):
            down.wait_event(ev_done[par])
            out[k].copy_(d_col[par], non_blocking=True)
            ev_d2h[par].record(down)
    torch.cuda.synchronize()
    for k in range(steps):
        assert torch.equal(out[k].view(torch.int32), refs[k % 2].view(torch.int32)), f"frame {k}"
