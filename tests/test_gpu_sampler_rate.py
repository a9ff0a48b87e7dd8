"""vct_sampler_rate: the cone tracer's sampler measured alone (the
denominator of the tracer's roofline) is at least as fast per sample as the
tracer, for every sampler, and the call validates its arguments."""

from __future__ import annotations

import pytest

from helpers import GpuScene
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def test_sampler_rate_bounds_the_tracer():
    import torch

    sc = scenes.cornell(seed=9, gbuffer=(640, 360))
    g = GpuScene(sc)
    ctx = api.Context(api.config_for(sc))
    with pytest.raises(L.VctError) as e:
        ctx.sampler_rate(L.VCT_FILTER_SOFTWARE)
    assert e.value.status == L.VCT_ERR_STATE  # no chain yet
    ctx.set_params(api.scene_params(sc))
    irr, spec, col, samples = g.new_outputs()
    ctx.enable_timers(True)
    for _ in range(3):
        samples.zero_()
        ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    trace_rate = int(samples.item()) / (ctx.timers()["render_ms"] * 1e-3)
    rates = {f: ctx.sampler_rate(f, 1 << 28) for f in (L.VCT_FILTER_SOFTWARE, L.VCT_FILTER_HYBRID,
                                                       L.VCT_FILTER_HARDWARE_LEVELS, L.VCT_FILTER_HARDWARE)}
    print("samples/s: trace", f"{trace_rate:.3e}", {k: f"{v:.3e}" for k, v in rates.items()})
    assert all(v > 0 for v in rates.values())
    assert rates[L.VCT_FILTER_SOFTWARE] > trace_rate
    with pytest.raises(L.VctError):
        ctx.sampler_rate(7)
