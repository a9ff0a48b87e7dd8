"""Generates the known-answer vectors in tests/golden/*.json.

The reference ships no tests, fixtures or golden outputs, so these vectors
are derived by hand from the GLSL semantics and written down here in closed
form with numpy only (no use of the oracle or the CUDA library):

  fp16.json          IEEE binary16 round-to-nearest-even (numpy float16).
  mvp.json           the per-axis voxelisation matrices of
                     src/Application.cpp:689-692 for the volume [-1,1]^3:
                     x: (x,y,z) -> (-z, y, -x), y: -> (x, -z, -y), z: -> (x, y, -z).
  quad_voxel.json    one z-facing quad (two triangles) through voxelize.geom/.frag
                     at 16^3: the pixel centres inside [-0.5,0.5]^2 (pixels
                     4..11) land in depth slice trunc(16*(z+1)/2); the shared
                     diagonal is covered exactly once (top-left rule); unlit
                     colour = albedo, normal (0,0,1) -> (0.5,0.5,1) in 16-bit
                     fixed point.
  tie_axis.json      a triangle whose summed normal has |nx| == |ny| falls to
                     the z projection (strict > in voxelize.geom:34-45); it is
                     edge-on there, so it yields no fragment.
  shadow_quad.json   the quad y=0, |x|,|z| <= 0.5 rendered into a 32^2 depth map
                     from a light looking down -y (ortho [-1,1]^2, depth 0..2):
                     depth 0.5 on texels 8..23 x 8..23, 1.0 (clear) elsewhere.
  inject_plane.json  injectRadiance.comp with a constant 0.5 depth map of 32^2
                     and the same light: texel (x,y) is sampled at its corner
                     (x/32, y/32), so x=0 or y=0 averages in the 1.0 border;
                     the lit voxels are the plane y=8 (all x,z) and the column
                     x=0, y=4, while row y=0 maps to z=16 (dropped).
  mip_point.json     a single voxel of value 1 at (5,6,7) in 16^3 propagates to
                     (2,3,3)=0.125, (1,1,1)=2^-6, (0,0,0) of levels 3 and 4 with
                     binary16 rounding at every level.
  trace_const.json   a 32^3 volume holding (0.5,0.5,0.5,0.5) at every level,
                     one pixel at the centre, normal +y: every diffuse cone
                     takes 5 samples before alpha >= 0.95, so each returns
                     rgb = a = 1 - 0.5^5 = 0.96875 and the weights sum to 1.

Run: python tests/golden/make_golden.py
"""

from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def dump(name, obj):
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(obj, f, indent=1, sort_keys=True)
        f.write("\n")


def fp16():
    vals = [0.0, -0.0, 1.0, -2.5, 0.1, 1.0 / 3.0, 65504.0, 65519.99, 65520.0, 1e6, 2.0 ** -14, 2.0 ** -24,
            2.0 ** -25, 3 * 2.0 ** -26, 2.0 ** -26, 0.5 + 2.0 ** -12, 0.5 + 3 * 2.0 ** -12, 1.0 + 2.0 ** -11,
            1.0 + 3 * 2.0 ** -11, 6.1e-5, 5.96e-8, 1234.567, -0.000123]
    rng = np.random.default_rng(0)
    vals += list(rng.uniform(-70000, 70000, 40)) + list(np.exp(rng.uniform(-20, 11, 40)))
    f32 = np.asarray(vals, dtype=np.float32)
    with np.errstate(over="ignore"):  # 65520 and 1e6 round to infinity
        f16 = f32.astype(np.float16)
    dump("fp16.json", {"f32_bits": f32.view(np.uint32).tolist(), "f16_bits": f16.view(np.uint16).tolist()})


def mvp():
    def cm(rows):
        return np.asarray(rows, dtype=np.float64).T.reshape(16).tolist()

    x = [[0, 0, -1, 0], [0, 1, 0, 0], [-1, 0, 0, 0], [0, 0, 0, 1]]
    y = [[1, 0, 0, 0], [0, 0, -1, 0], [0, -1, 0, 0], [0, 0, 0, 1]]
    z = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, -1, 0], [0, 0, 0, 1]]
    dump("mvp.json", {"vmax": 1.0, "dim": 16, "mvp": cm(x) + cm(y) + cm(z)})


def quad_voxel():
    zq = 0.03
    p = [[-0.5, -0.5, zq], [0.5, -0.5, zq], [0.5, 0.5, zq], [-0.5, 0.5, zq]]
    tris = [p[0] + p[1] + p[2], p[0] + p[2] + p[3]]
    nrm = [[0, 0, 1] * 3] * 2
    alb = [[0.25, 0.5, 0.75]] * 2
    N = 16
    iz = int(np.floor(N * (zq + 1.0) / 2.0))  # 8
    q = lambda v: int(np.rint(v * 65535.0))  # noqa: E731
    sums = [q(0.25), q(0.5), q(0.75), q(0.5), q(0.5), q(1.0)]
    voxels = [[x, y, iz] for y in range(4, 12) for x in range(4, 12)]
    dump("quad_voxel.json", {"dim": N, "vmax": 1.0, "positions": tris, "normals": nrm, "albedo": alb,
                             "voxels": voxels, "count": 1, "sums": sums, "total_fragments": 64})


def tie_axis():
    # Plane x = y: vertex normals (1,-1,0)/sqrt2 sum to |nx| == |ny|.
    s = 1 / np.sqrt(2)
    tri = [0.1, 0.1, -0.4, -0.3, -0.3, 0.2, 0.4, 0.4, 0.3]
    dump("tie_axis.json", {"dim": 16, "vmax": 1.0, "positions": [tri], "normals": [[s, -s, 0] * 3],
                           "albedo": [[1, 1, 1]], "total_fragments": 0})


def light_down():
    """ls = ortho(-1,1,-1,1,0,2) * lookAt((0,1,0),(0,0,0),(0,0,-1)): ndc = (x, -z, -y)."""
    m = np.array([[1, 0, 0, 0], [0, 0, -1, 0], [0, -1, 0, 0], [0, 0, 0, 1]], dtype=np.float64)
    return m.T.reshape(16).tolist(), np.linalg.inv(m).T.reshape(16).tolist()


def shadow_quad():
    ls, _ = light_down()
    W = 32
    depth = np.ones((W, W))
    depth[8:24, 8:24] = 0.5
    tris = [[-0.5, 0, -0.5, 0.5, 0, -0.5, 0.5, 0, 0.5], [-0.5, 0, -0.5, 0.5, 0, 0.5, -0.5, 0, 0.5]]
    dump("shadow_quad.json", {"size": W, "ls": ls, "positions": tris, "depth": depth.reshape(-1).tolist()})


def inject_plane():
    ls, lsi = light_down()
    W, N = 32, 16
    lit = set()
    for y in range(W):
        for x in range(W):
            d = 0.5 if (x >= 1 and y >= 1) else (0.875 if (x == 0 and y == 0) else 0.75)
            px, pz, py = x / 16.0 - 1.0, 1.0 - y / 16.0, 1.0 - 2.0 * d
            v = [int(np.trunc(N * (c + 1.0) / 2.0)) for c in (px, py, pz)]
            if all(0 <= c < N for c in v):
                lit.add(tuple(v))
    dump("inject_plane.json", {"size": W, "dim": N, "vmax": 1.0, "ls": ls, "ls_inverse": lsi, "depth": 0.5,
                               "color": [0.25, 0.5, 0.75, 0.5], "lit_voxels": sorted(list(v) for v in lit)})


def mip_point():
    N, levels = 16, 5
    vol = np.zeros((N, N, N), dtype=np.float16)
    vol[7, 6, 5] = 1.0  # [z, y, x]
    expect = []
    cur = vol
    for l in range(1, levels):
        D = cur.shape[0] // 2
        nxt = cur.astype(np.float32).reshape(D, 2, D, 2, D, 2).sum(axis=(1, 3, 5)) * np.float32(0.125)
        cur = nxt.astype(np.float16)
        nz = np.argwhere(cur != 0)
        expect.append([[int(i) for i in k[::-1]] + [float(cur[tuple(k)])] for k in nz])
    dump("mip_point.json", {"dim": N, "levels": levels, "voxel": [5, 6, 7], "expect": expect})


def trace_const():
    dump("trace_const.json", {"dim": 32, "value": 0.5, "normal": [0, 1, 0], "position": [0, 0, 0],
                              "irradiance": [0.96875, 0.96875, 0.96875, 0.96875], "samples_per_cone": 5})


if __name__ == "__main__":
    fp16()
    mvp()
    quad_voxel()
    tie_axis()
    shadow_quad()
    inject_plane()
    mip_point()
    trace_const()
    print("golden vectors written to", HERE)
