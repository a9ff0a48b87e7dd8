"""phong.frag's full composite (vct_shade): direct lighting of every light
(Cook-Torrance or Blinn-Phong, point-light attenuation, PCF shadows) plus the
indirect term of the cone trace, occlusion and the tone map, against the
CPU restatement (powf vs std::pow differ by rounding: relative L2 <= 1e-5)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from helpers import GpuScene, rel_l2, rgb
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["tiny", "cornell"])
def traced(request):
    import torch

    sc = scenes.tiny(seed=4, dim=32, shadow=256, gbuffer=(200, 120)) if request.param == "tiny" else \
        scenes.cornell(seed=9, gbuffer=(320, 180))
    g = GpuScene(sc)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc))
    irr, spec, col, samples = g.new_outputs()
    ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    return sc, g, ctx, irr, spec


@pytest.mark.parametrize("cook", [1, 0], ids=["cooktorrance", "blinnphong"])
@pytest.mark.parametrize("indirect", [1, 0], ids=["indirect", "direct_only"])
@pytest.mark.parametrize("post", [1, 0], ids=["tonemap", "linear"])
def test_shade_matches_oracle(traced, cook, indirect, post):
    import torch

    sc, g, ctx, irr, spec = traced
    p = api.scene_params(sc, cooktorrance=cook, enable_indirect=indirect, enable_postprocess=post)
    ctx.set_params(p)
    W, H = sc.gbuffer_size
    out = torch.zeros(W * H * 4, device="cuda")
    ctx.shade(g.gb, sc.eye, g.lights, g.shadow, out, irr, spec)
    torch.cuda.synchronize()
    sm, gbuf = g.host_inputs()
    ref = O.shade(sc, gbuf, sm, irr.cpu().numpy(), spec.cpu().numpy(), cooktorrance=cook, enable_indirect=indirect,
                  enable_postprocess=post)
    got = out.cpu().numpy()
    assert np.abs(rgb(got)).sum() > 0
    e = rel_l2(rgb(got), rgb(ref))
    assert e <= 1e-5, e
    cov = gbuf[0].reshape(-1, 4)[:, 3] != 0
    assert np.all(got.reshape(-1, 4)[cov, 3] == 1.0) and np.all(got.reshape(-1, 4)[~cov] == 0.0)


def test_shade_direct_terms_switch(traced):
    """Direct diffuse and specular switched off leave the ambient / indirect
    composite the trace itself writes."""
    import torch

    sc, g, ctx, irr, spec = traced
    ctx.set_params(api.scene_params(sc, enable_diffuse=0, enable_specular=0))
    W, H = sc.gbuffer_size
    out = torch.zeros(W * H * 4, device="cuda")
    col = torch.zeros(W * H * 4, device="cuda")
    ctx.shade(g.gb, sc.eye, g.lights, g.shadow, out, irr, spec)
    ctx.trace(g.gb, sc.eye, api.trace_out(color=col))
    torch.cuda.synchronize()
    assert rel_l2(rgb(out.cpu().numpy()), rgb(col.cpu().numpy())) <= 1e-6
