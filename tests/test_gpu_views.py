"""vct_trace_views: several viewpoints of one set of volumes traced by one
launch per 8 viewpoints, each view equal, bit for bit, to its own vct_trace
call: the trace outputs and the sample counters, for 9 views of different
G-buffer sizes (two launches), with the exact and the hybrid samplers and
with the perspective warp."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import GpuScene
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _views(sc, g, n):
    import torch

    out = []
    for k in range(n):
        W, H = (320, 180) if k % 3 else (256, 160)
        v = scenes.viewpoint(sc, k, n)
        v.gbuffer_size = (W, H)
        keys = torch.empty(W * H, dtype=torch.int64, device="cuda")
        gp, gn, ga = (torch.empty(W * H * 4, dtype=torch.float32, device="cuda") for _ in range(3))
        api.render_gbuffer(g.tris, v, keys, gp, gn, ga)
        out.append((v, (gp, gn, ga), api.gbuffer(gp, gn, ga, W, H)))
    return out


@pytest.mark.parametrize("filt,warp", [(L.VCT_FILTER_SOFTWARE, L.VCT_WARP_NONE), (L.VCT_FILTER_HYBRID, L.VCT_WARP_NONE),
                                       (L.VCT_FILTER_SOFTWARE, L.VCT_WARP_PERSPECTIVE)],
                         ids=["software", "hybrid", "perspective"])
def test_trace_views_equal_single_traces(filt, warp):
    import torch

    sc = scenes.cornell(seed=9, gbuffer=(320, 180))
    g = GpuScene(sc)
    views = _views(sc, g, 9)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc, trace_filter=filt, warp_mode=warp))
    ctx.voxelize(g.tris, g.lights, g.shadow, sc.eye)
    ctx.inject(g.shadow, sc.eye)
    ctx.build_mips()

    def outs_for(v):
        W, H = v.gbuffer_size
        t = [torch.zeros(W * H * 4, device="cuda") for _ in range(3)] + [torch.zeros(1, dtype=torch.int64,
                                                                                     device="cuda")]
        return t, api.trace_out(*t)

    single = []
    for v, _, gb in views:
        t, o = outs_for(v)
        ctx.trace(gb, v.eye, o)
        single.append(t)
    multi = [outs_for(v) for v, _, _ in views]
    ctx.trace_views([gb for _, _, gb in views], [v.eye for v, _, _ in views], [o for _, o in multi])
    torch.cuda.synchronize()
    for k, (a, (b, _)) in enumerate(zip(single, multi)):
        for x, y in zip(a, b):
            assert torch.equal(x.view(torch.int32) if x.dtype == torch.float32 else x,
                               y.view(torch.int32) if y.dtype == torch.float32 else y), f"view {k}"
        assert int(a[3].item()) > 0
    # no views: nothing to do
    ctx.trace_views([], [], [])
    ctx.close()
