"""Shared helpers of the parity tests: upload a scene, run GPU stages through
the C ABI, run the oracle on the same inputs."""

from __future__ import annotations

import numpy as np

import oracle as O
from vct_gb300 import _lib as L
from vct_gb300 import api


def u16(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint16)


def u32(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)


class GpuScene:
    """A scene's triangles, shadow map and G-buffer resident on cuda:0."""

    def __init__(self, sc, shadowmap=None, gbuf=None, device="cuda:0"):
        import torch

        self.sc = sc
        self.dev = device
        self.pos = torch.from_numpy(sc.positions).to(device)
        self.nrm = torch.from_numpy(sc.normals).to(device)
        self.alb = torch.from_numpy(sc.albedo).to(device)
        self.tris = api.triangles(self.pos, self.nrm, self.alb)
        W, H = sc.shadow_size
        if shadowmap is None:
            self.sm = torch.empty(W * H, dtype=torch.float32, device=device)
            api.render_shadowmap(self.tris, sc, self.sm)
        else:
            self.sm = torch.from_numpy(np.ascontiguousarray(shadowmap, dtype=np.float32)).to(device)
        GW, GH = sc.gbuffer_size
        if gbuf is None:
            self.keys = torch.empty(GW * GH, dtype=torch.int64, device=device)
            self.gpos, self.gnrm, self.galb = (torch.empty(GW * GH * 4, dtype=torch.float32, device=device)
                                               for _ in range(3))
            api.render_gbuffer(self.tris, sc, self.keys, self.gpos, self.gnrm, self.galb)
        else:
            self.gpos, self.gnrm, self.galb = (torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in gbuf)
        self.lights = api.light_array(sc.lights)
        self.shadow = api.shadow_desc(sc, self.sm)
        self.gb = api.gbuffer(self.gpos, self.gnrm, self.galb, GW, GH)

    def host_inputs(self):
        return (self.sm.cpu().numpy(), (self.gpos.cpu().numpy(), self.gnrm.cpu().numpy(), self.galb.cpu().numpy()))

    def new_outputs(self):
        import torch

        GW, GH = self.sc.gbuffer_size
        irr, spec, col = (torch.zeros(GW * GH * 4, dtype=torch.float32, device=self.dev) for _ in range(3))
        samples = torch.zeros(1, dtype=torch.int64, device=self.dev)
        return irr, spec, col, samples


def split_records(rec, occ):
    """GPU accumulator records -> (count, SoA sums, occupancy bools) as the
    oracle lays them out."""
    r = u32(rec).reshape(-1, 8)
    count = np.ascontiguousarray(r[:, 0])
    sums = np.ascontiguousarray(r[:, 1:7].T).reshape(-1)
    bits = np.unpackbits(u32(occ).view(np.uint8), bitorder="little")[: r.shape[0]].astype(bool)
    return count, sums, bits, r[:, 7]


def read_chain(ctx, volume=L.VCT_VOLUME_RADIANCE) -> np.ndarray:
    return np.concatenate([u16(ctx.read_volume(volume, l)) for l in range(ctx.levels)])


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def rgb(x) -> np.ndarray:
    return np.asarray(x).reshape(-1, 4)[:, :3]
