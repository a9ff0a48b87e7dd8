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
