"""The learned path against the oracle: cheap quarter-resolution features,
the 16-cone reference trace (against FP64), feature rows, the fused learned
trace against the network run on those rows, the per-tile fallback, and
what a trained network gains over the cheap trace without it."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from helpers import GpuScene, read_chain
from vct_gb300 import _lib as L
from vct_gb300 import api, learned, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def frame():
    import torch

    sc = scenes.cornell(seed=4, gbuffer=(322, 182))
    g = GpuScene(sc)
    ctx = api.Context(api.config_for(sc))
    ctx.set_params(api.scene_params(sc))
    irr, spec, col, samples = g.new_outputs()
    ctx.frame(g.tris, g.lights, g.shadow, sc.eye, g.gb, api.trace_out(irr, spec, col, samples))
    torch.cuda.synchronize()
    chain = read_chain(ctx)
    W, H = sc.gbuffer_size
    q = torch.empty(((W + 3) // 4) * ((H + 3) // 4) * 32, dtype=torch.int16, device="cuda")
    api.learned_features(ctx, g.gb, sc.eye, q)
    torch.cuda.synchronize()
    host = dict(gpos=g.gpos.cpu().numpy(), gnrm=g.gnrm.cpu().numpy(), galb=g.galb.cpu().numpy())
    return sc, g, ctx, chain, q, host


def _bf16(x):
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    return ((((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32)).view(np.float32)


def test_cheap_features_match_oracle(frame):
    import torch

    sc, g, ctx, chain, q, host = frame
    got = q.view(torch.bfloat16).float().cpu().numpy().reshape(-1, 32)
    ref = _bf16(O.learned_features(sc, chain, host["gpos"], host["gnrm"]))
    assert np.count_nonzero(ref) > 0.3 * ref.size
    # fp32 trilinear rounding may differ by an ulp, which can move a BF16 rounding by one BF16 ulp
    close = np.abs(got - ref) <= 2.0 ** -7 * np.abs(ref) + 1e-30
    assert close.mean() == 1.0, close.mean()
    assert (got == ref).mean() > 0.99


def test_reference16_matches_fp64_oracle(frame):
    import torch

    sc, g, ctx, chain, q, host = frame
    W, H = sc.gbuffer_size
    out = torch.zeros(W * H * 4, device="cuda")
    api.trace_reference16(ctx, g.gb, sc.eye, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(-1, 4)
    rng = np.random.default_rng(0)
    pix = np.sort(rng.choice(W * H, 3000, replace=False)).astype(np.int32)
    r64, _ = O.trace_reference16(sc, chain, host["gpos"], host["gnrm"], pix, precision=64, nthreads=8)
    r32, _ = O.trace_reference16(sc, chain, host["gpos"], host["gnrm"], pix, precision=32, nthreads=8)
    err64 = np.linalg.norm(got[pix, :3] - r64[:, :3]) / np.linalg.norm(r64[:, :3])
    err32 = np.linalg.norm(got[pix, :3] - r32[:, :3]) / np.linalg.norm(r32[:, :3])
    print(f"16-cone irradiance rel L2: vs fp64 {err64:.2e}, vs fp32 {err32:.2e}")
    assert err64 < 1e-3 and err32 < 1e-4
    assert np.all(got[:, 3] == 0.0)


def test_rows_are_the_pixel_features(frame):
    import torch

    sc, g, ctx, chain, q, host = frame
    W, H = sc.gbuffer_size
    pix = torch.arange(0, W * H, 7, dtype=torch.int32, device="cuda")
    rows = torch.empty(pix.numel(), 42, device="cuda")
    api.learned_rows(ctx, g.gb, sc.eye, q, pix, rows)
    r = rows.cpu().numpy()
    p = pix.cpu().numpy()
    gp = host["gpos"].reshape(-1, 4)[p]
    gn = host["gnrm"].reshape(-1, 4)[p, :3]
    ga = host["galb"].reshape(-1, 4)[p, :3]
    cov = gp[:, 3] != 0
    assert np.all(r[~cov] == 0)
    qf = q.view(torch.bfloat16).float().cpu().numpy().reshape(-1, 32)
    blk = (p // W // 4) * ((W + 3) // 4) + (p % W) // 4
    assert np.array_equal(r[cov, :32], qf[blk[cov]])
    n = gn / np.maximum(np.linalg.norm(gn, axis=1, keepdims=True), 1e-30)
    d = gp[:, :3] - sc.eye[None]
    dist = np.linalg.norm(d, axis=1)
    assert np.allclose(r[cov, 32:35], n[cov], atol=8e-3)
    assert np.allclose(r[cov, 35], dist[cov] / (2 * sc.vmax), rtol=8e-3)
    assert np.allclose(r[cov, 36:39], ga[cov], rtol=8e-3, atol=1e-6)
    # near-field radiance: level 1 sampled trilinearly two voxels above the surface
    S = sc.dim // 2
    lvl = ctx.read_volume(L.VCT_VOLUME_RADIANCE, 1).view(torch.float16).float().cpu().numpy().reshape(S, S, S, 4)
    vp = (gp[:, :3] + sc.vmax) / (2 * sc.vmax) + n * (2.0 / sc.dim)
    u = vp * S - 0.5
    i0 = np.floor(u).astype(int)
    a = u - i0
    near = np.zeros((len(p), 4))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                ix, iy, iz = i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz
                ok = (ix >= 0) & (iy >= 0) & (iz >= 0) & (ix < S) & (iy < S) & (iz < S)
                w = (a[:, 0] if dx else 1 - a[:, 0]) * (a[:, 1] if dy else 1 - a[:, 1]) * (a[:, 2] if dz else 1 - a[:, 2])
                near += (w * ok)[:, None] * lvl[iz.clip(0, S - 1), iy.clip(0, S - 1), ix.clip(0, S - 1)]
    inside = np.all((vp >= 0) & (vp <= 1), axis=1)
    near[~inside] = 0
    assert np.allclose(r[cov, 39:42], near[cov, :3], rtol=8e-3, atol=1e-4)
    assert np.array_equal(r, _bf16(r))  # exactly the BF16 inputs of the network


def test_learned_trace_is_the_network_on_the_rows_and_falls_back_per_tile(frame):
    import torch

    sc, g, ctx, chain, q, host = frame
    W, H = sc.gbuffer_size
    mlp = api.Mlp(seed=1)
    pix = torch.arange(W * H, dtype=torch.int32, device="cuda")
    rows = torch.empty(W * H, 42, device="cuda")
    api.learned_rows(ctx, g.gb, sc.eye, q, pix, rows)
    net4 = torch.empty(W * H, 4, device="cuda")
    mlp.forward(rows, net4)
    net = net4[:, :3]
    out = torch.zeros(W * H * 4, device="cuda")
    api.learned_trace(ctx, mlp, g.gb, sc.eye, out, float("inf"))
    torch.cuda.synchronize()
    cov = torch.from_numpy(host["gpos"].reshape(-1, 4)[:, 3] != 0).cuda()
    o = out.view(-1, 4)
    assert torch.equal(o[cov, :3], net[cov])
    assert torch.all(o[~cov] == 0)
    # with the fallback: listed tiles hold the 16-cone trace, the others the network
    ref = torch.zeros(W * H * 4, device="cuda")
    api.trace_reference16(ctx, g.gb, sc.eye, ref)
    st = api.learned_trace(ctx, mlp, g.gb, sc.eye, out, 0.02, want_stats=True)
    tiles_x, tiles_y = (W + 15) // 16, (H + 15) // 16
    assert st["tiles"] == tiles_x * tiles_y
    assert st["fallback_tiles"] > 0  # an untrained network is far off
    o = out.view(H, W, 4).cpu().numpy()
    r = ref.view(H, W, 4).cpu().numpy()
    nn = torch.where(cov[:, None], net, torch.zeros_like(net)).view(H, W, 3).cpu().numpy()
    n_ref = n_net = 0
    for ty in range(tiles_y):
        for tx in range(tiles_x):
            sl = (slice(16 * ty, 16 * ty + 16), slice(16 * tx, 16 * tx + 16))
            if np.array_equal(o[sl][..., :3], r[sl][..., :3]):
                n_ref += 1
            else:
                assert np.array_equal(o[sl][..., :3], nn[sl]), (tx, ty)
                n_net += 1
    assert n_ref >= st["fallback_tiles"]


def test_pixel_fallback_retraces_exactly_the_flagged_pixels(frame):
    """vct_learned_trace_pixels: the covered pixels whose error estimate (the
    network's fourth output, as vct_mlp_forward gives it on the same rows)
    exceeds threshold x the RMS of the network's irradiance over covered
    pixels hold the 16-cone trace bit for bit; every other pixel holds the
    network's irradiance; the reported count is their number.  (The RMS is
    summed on the device in an arbitrary order, so estimates within 1e-4 of
    the bound may go either way.)"""
    import torch

    sc, g, ctx, chain, q, host = frame
    W, H = sc.gbuffer_size
    mlp = api.Mlp(seed=2)
    w = mlp.params()
    w[api.Mlp.NPARAMS - 1] += 4.0  # the error estimate's bias: every estimate positive
    mlp.set_params(w)
    pix = torch.arange(W * H, dtype=torch.int32, device="cuda")
    rows = torch.empty(W * H, 42, device="cuda")
    api.learned_rows(ctx, g.gb, sc.eye, q, pix, rows)
    net = torch.empty(W * H, 4, device="cuda")
    mlp.forward(rows, net)
    ref = torch.zeros(W * H * 4, device="cuda")
    api.trace_reference16(ctx, g.gb, sc.eye, ref)
    cov = torch.from_numpy(host["gpos"].reshape(-1, 4)[:, 3] != 0).cuda()
    rms = float(net[cov, :3].double().pow(2).sum(1).mean().sqrt())
    thr = float(net[cov, 3].double().median()) / rms
    out = torch.full((W * H * 4,), -1.0, device="cuda")
    n = api.learned_trace_pixels(ctx, mlp, g.gb, sc.eye, out, thr, want_count=True)
    est, bound = net[:, 3].double(), thr * rms
    flagged = cov & (est > bound * (1 + 1e-4))
    kept = cov & (est < bound * (1 - 1e-4))
    assert 0 < int(flagged.sum()) <= n <= int(flagged.sum()) + int((cov & ~flagged & ~kept).sum())
    assert int(kept.sum()) > 0
    o, r = out.view(-1, 4), ref.view(-1, 4)
    assert torch.equal(o[flagged], r[flagged])
    assert torch.equal(o[kept, :3], net[kept, :3]) and torch.all(o[kept, 3] == 0)
    assert torch.all(o[~cov] == 0)
    # no bound: the network alone, the same image as vct_learned_trace without fallback
    plain = torch.zeros(W * H * 4, device="cuda")
    api.learned_trace(ctx, mlp, g.gb, sc.eye, plain, float("inf"))
    assert api.learned_trace_pixels(ctx, mlp, g.gb, sc.eye, out, float("inf"), want_count=True) == 0
    assert torch.equal(out, plain)


def test_trained_network_beats_the_cheap_trace():
    """A short training run on family scenes (128^3, 480x270): on held-out
    scenes the network's irradiance error is well below that of the two cheap
    cones used directly, and the per-tile fallback cuts it further."""
    kw = dict(dim=128, shadow=1024, gbuffer=(480, 270), n_boxes=1024, n_cyl=16, cyl_segments=256)
    state = learned.FrameState(128, (480, 270), 1024)
    rows, targets = learned.build_dataset(state, list(range(24)), 8192, kw)
    mlp = api.Mlp(seed=0)
    hist = learned.train(mlp, rows, targets, epochs=30, batch=4096, lr=3e-3)
    print("loss per epoch", [round(h, 6) for h in hist])
    assert hist[-1] < 0.25 * hist[0], hist
    ev = learned.evaluate(mlp, state, [1000, 1001, 1002], kw, threshold=0.02)
    net, cheap, fb = np.mean(ev["network"]), np.mean(ev["cheap"]), np.mean(ev["with_fallback"])
    print(f"held-out rel L2: network {net:.4f}, with fallback {fb:.4f}, cheap {cheap:.4f}; "
          f"fallback tiles {np.mean(ev['fallback_fraction']):.3f}")
    assert net < 0.7 * cheap
    assert fb < 0.5 * net
