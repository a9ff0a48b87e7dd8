"""Learned indirect light: data generation, training and evaluation of the
MLP that turns the cheap two-cone quarter-resolution trace plus G-buffer
features into the 16-cone full-resolution irradiance.

Everything runs on the GPU through the C ABI (include/vct.h): scenes are
voxelised, injected and filtered by the frame kernels, the 16-cone targets
come from vct_trace_reference16, feature rows from vct_learned_rows, and the
network (irradiance and an estimate of its own error, which drives the
per-pixel fallback) trains with the tensor-core kernels behind
vct_mlp_train_step.
torch only allocates device memory and draws random permutations.

    python -m vct_gb300.learned train --scenes 2000 --holdout 200 --out vct_gb300/weights/learned_mlp
"""

from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import _lib as L
from . import api, scenes

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights", "learned_mlp")
CHEAP = 32
FEATURES = 42


class FrameState:
    """Device buffers of one scene configuration (grid, G-buffer and shadow
    map sizes), reused for every scene of a family."""

    def __init__(self, dim: int, gbuffer: tuple, shadow: int, device: int = 0, vmax: float = 1.0):
        import torch

        self.dev = f"cuda:{device}"
        self.W, self.H = gbuffer
        self.wq, self.hq = (self.W + 3) // 4, (self.H + 3) // 4
        probe = scenes.tiny()
        probe.dim, probe.vmax = dim, vmax
        self.ctx = api.Context(api.config_for(probe, device=device))
        P = self.W * self.H
        self.keys = torch.empty(P, dtype=torch.int64, device=self.dev)
        self.gpos, self.gnrm, self.galb = (torch.empty(P * 4, dtype=torch.float32, device=self.dev) for _ in range(3))
        self.sm = torch.empty(shadow * shadow, dtype=torch.float32, device=self.dev)
        self.qfeat = torch.empty(self.wq * self.hq * CHEAP, dtype=torch.int16, device=self.dev)
        self.ref = torch.empty(P * 4, dtype=torch.float32, device=self.dev)
        self.out = torch.empty(P * 4, dtype=torch.float32, device=self.dev)
        self.gb = api.gbuffer(self.gpos, self.gnrm, self.galb, self.W, self.H)
        self.sc = None

    def load(self, sc, stream=None):
        """Uploads a scene, renders its shadow map and G-buffer and builds its
        radiance chain (voxelise, normalise, inject, mips)."""
        import torch

        assert sc.gbuffer_size == (self.W, self.H)
        self.pos, self.nrm, self.alb = (torch.from_numpy(a).to(self.dev) for a in (sc.positions, sc.normals, sc.albedo))
        tris = api.triangles(self.pos, self.nrm, self.alb)
        api.render_shadowmap(tris, sc, self.sm, stream)
        api.render_gbuffer(tris, sc, self.keys, self.gpos, self.gnrm, self.galb, stream)
        self.ctx.set_params(api.scene_params(sc))
        shadow = api.shadow_desc(sc, self.sm)
        self.ctx.voxelize(tris, api.light_array(sc.lights), shadow, sc.eye, stream)
        self.ctx.inject(shadow, sc.eye, stream)
        self.ctx.build_mips(stream=stream)
        self.sc = sc

    def features(self, stream=None):
        api.learned_features(self.ctx, self.gb, self.sc.eye, self.qfeat, stream)

    def reference(self, out=None, stream=None):
        api.trace_reference16(self.ctx, self.gb, self.sc.eye, self.ref if out is None else out, stream)

    def covered(self):
        return self.gpos.view(-1, 4)[:, 3] != 0

    def rows(self, pixels, rows_out, stream=None):
        api.learned_rows(self.ctx, self.gb, self.sc.eye, self.qfeat, pixels, rows_out, stream)

    def cheap_irradiance(self):
        """The method without the network: the two cheap cones' composited
        radiance (their last feature checkpoint, level 8), averaged, each
        pixel taking its 4x4 block's value.  (H * W, 3) torch tensor."""
        import torch

        f = self.qfeat.view(torch.bfloat16).float().view(-1, 2, 4, 4)  # block, cone, checkpoint, rgba
        irr = f[:, :, 3, :3].mean(1)
        ys = torch.arange(self.H, device=f.device) // 4
        xs = torch.arange(self.W, device=f.device) // 4
        blk = (ys[:, None] * self.wq + xs[None, :]).reshape(-1)
        return irr[blk] * self.covered()[:, None]


def rel_l2(pred, truth, mask) -> float:
    """Relative L2 error of RGB over the covered pixels."""
    d = (pred - truth)[mask]
    t = truth[mask]
    return float(d.double().norm() / max(float(t.double().norm()), 1e-30))


def _scene_worker(args):
    seed, kw = args
    return scenes.large_family(seed, **kw)


def scene_stream(seeds, kw, workers: int = 0):
    """Yields scenes of the family; with workers > 0 they are generated by a
    spawn-started process pool ahead of use."""
    if workers <= 0:
        for s in seeds:
            yield scenes.large_family(s, **kw)
        return
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        yield from pool.imap(_scene_worker, [(s, kw) for s in seeds], chunksize=2)


def build_dataset(state: FrameState, seeds, pixels_per_scene: int, kw: dict, workers: int = 0, log=None):
    """Rows (N x 42) and 16-cone targets (N x 3) of random covered pixels of
    each scene, on the device."""
    import torch

    n_max = len(seeds) * pixels_per_scene
    rows = torch.empty(n_max, FEATURES, dtype=torch.float32, device=state.dev)
    targets = torch.empty(n_max, 3, dtype=torch.float32, device=state.dev)
    n = 0
    gen = torch.Generator(device=state.dev)
    gen.manual_seed(1234)
    t0 = time.time()
    for i, sc in enumerate(scene_stream(seeds, kw, workers)):
        state.load(sc)
        state.features()
        state.reference()
        cov = torch.nonzero(state.covered()).view(-1).to(torch.int32)
        if cov.numel() == 0:
            continue
        k = min(pixels_per_scene, cov.numel())
        pick = cov[torch.randperm(cov.numel(), device=state.dev, generator=gen)[:k]].contiguous()
        state.rows(pick, rows[n:n + k])
        targets[n:n + k] = state.ref.view(-1, 4)[pick.long(), :3]
        n += k
        if log and (i + 1) % 100 == 0:
            log(f"dataset: {i + 1}/{len(seeds)} scenes, {n} rows, {time.time() - t0:.1f}s")
    torch.cuda.synchronize()
    return rows[:n], targets[:n]


def train(mlp: api.Mlp, rows, targets, epochs: int = 20, batch: int = 16384, lr: float = 2e-3, lr_min: float = 2e-5,
          seed: int = 0, log=None):
    """Adam with a cosine learning-rate schedule over shuffled minibatches;
    returns the loss history (one mean per epoch)."""
    import torch

    n = rows.shape[0]
    steps_per_epoch = max(1, n // batch)
    total = epochs * steps_per_epoch
    gen = torch.Generator(device=rows.device)
    gen.manual_seed(seed)
    loss = torch.zeros(steps_per_epoch, dtype=torch.float32, device=rows.device)
    hist = []
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(n, device=rows.device, generator=gen).to(torch.int32)
        for s in range(steps_per_epoch):
            t = step / max(1, total - 1)
            cur = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * t))
            mlp.train_step(rows, targets, perm[s * batch:(s + 1) * batch], batch, cur, loss[s:s + 1])
            step += 1
        hist.append(float(loss.mean()))
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {hist[-1]:.6g}")
    return hist


# Per-pixel fallback bounds (error estimate / the frame's RMS irradiance) evaluated on held-out scenes.
PIXEL_THRESHOLDS = (0.02, 0.03, 0.05, 0.1, 0.2, 0.5)


def evaluate(mlp: api.Mlp, state: FrameState, seeds, kw: dict, threshold: float = 0.02, workers: int = 0,
             log=None, pixel_thresholds=PIXEL_THRESHOLDS) -> dict:
    """Per held-out scene: relative L2 irradiance error of the network alone,
    of the network with the per-tile fallback, of the network with the
    per-pixel fallback at each bound, and of the cheap two-cone estimate, all
    against the 16-cone trace; plus the fallback fractions (of tiles, and of
    covered pixels)."""
    res = {"network": [], "with_fallback": [], "cheap": [], "fallback_fraction": [], "est_tile_error": []}
    for t in pixel_thresholds:
        res[f"pixel_{t}"] = []
        res[f"pixel_{t}_fraction"] = []
    for i, sc in enumerate(scene_stream(seeds, kw, workers)):
        state.load(sc)
        state.reference()
        state.features()
        mask = state.covered()
        ncov = max(1, int(mask.sum()))
        truth = state.ref.view(-1, 4)[:, :3]
        api.learned_trace(state.ctx, mlp, state.gb, sc.eye, state.out, float("inf"))
        res["network"].append(rel_l2(state.out.view(-1, 4)[:, :3], truth, mask))
        st = api.learned_trace(state.ctx, mlp, state.gb, sc.eye, state.out, threshold, want_stats=True)
        res["with_fallback"].append(rel_l2(state.out.view(-1, 4)[:, :3], truth, mask))
        res["fallback_fraction"].append(st["fallback_tiles"] / st["tiles"])
        res["est_tile_error"].append(st["mean_tile_error"])
        for t in pixel_thresholds:
            n = api.learned_trace_pixels(state.ctx, mlp, state.gb, sc.eye, state.out, t, want_count=True)
            res[f"pixel_{t}"].append(rel_l2(state.out.view(-1, 4)[:, :3], truth, mask))
            res[f"pixel_{t}_fraction"].append(n / ncov)
        res["cheap"].append(rel_l2(state.cheap_irradiance(), truth, mask))
        if log and (i + 1) % 50 == 0:
            log(f"eval: {i + 1}/{len(seeds)}: network {np.mean(res['network']):.4f} fallback "
                f"{np.mean(res['with_fallback']):.4f} cheap {np.mean(res['cheap']):.4f}")
    return {k: [float(x) for x in v] for k, v in res.items()}


def save(mlp: api.Mlp, path: str, report: dict):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    mlp.params().astype("<f4").tofile(path + ".f32")
    with open(path + ".json", "w") as f:
        json.dump(report, f, indent=1)


def load_params(path: str = WEIGHTS) -> np.ndarray | None:
    p = path + ".f32"
    if not os.path.exists(p):
        return None
    a = np.fromfile(p, dtype="<f4")
    return a if a.size == api.Mlp.NPARAMS else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--scenes", type=int, default=2000)
    ap.add_argument("--holdout", type=int, default=200)
    ap.add_argument("--pixels", type=int, default=8192, help="training pixels per scene")
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--dim", type=int, default=256)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--shadow", type=int, default=2048)
    ap.add_argument("--threshold", type=float, default=0.02)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    args = ap.parse_args()
    import torch

    def log(msg):
        print(msg, flush=True)

    kw = dict(dim=args.dim, shadow=args.shadow, gbuffer=(args.width, args.height))
    train_seeds = list(range(args.seed, args.seed + args.scenes))
    hold_seeds = list(range(10_000_000 + args.seed, 10_000_000 + args.seed + args.holdout))
    state = FrameState(args.dim, (args.width, args.height), args.shadow)
    t0 = time.time()
    rows, targets = build_dataset(state, train_seeds, args.pixels, kw, args.workers, log)
    t_data = time.time() - t0
    log(f"dataset: {rows.shape[0]} rows in {t_data:.1f}s")
    mlp = api.Mlp(seed=args.seed)
    t0 = time.time()
    hist = train(mlp, rows, targets, args.epochs, args.batch, args.lr, log=log)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    del rows, targets
    ev = evaluate(mlp, state, hold_seeds, kw, args.threshold, args.workers, log)
    report = {
        "family": "large plain frame family (large_family): 262,144 tris, orbit camera",
        "grid": args.dim, "gbuffer": [args.width, args.height], "train_scenes": args.scenes,
        "holdout_scenes": args.holdout, "pixels_per_scene": args.pixels, "epochs": args.epochs,
        "batch": args.batch, "lr": args.lr, "loss_history": hist, "dataset_s": round(t_data, 1),
        "train_s": round(t_train, 1), "threshold": args.threshold,
        "holdout_rel_l2": {k: float(np.mean(v)) for k, v in ev.items()},
        "holdout_rel_l2_max": {k: float(np.max(v)) for k, v in ev.items()},
    }
    save(mlp, args.out, report)
    log(json.dumps(report["holdout_rel_l2"]))


if __name__ == "__main__":
    main()
