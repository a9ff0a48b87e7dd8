"""Seeded synthetic scenes for the VCT hot path.

The reference renders Sponza (missing from its repository); the benchmark
configurations instead name seeded synthetic scenes, generated here with
numpy only (deterministic for a given seed):

  cornell  - 5 axis-aligned wall quads (an open-top box, 10 triangles) with a
             per-wall albedo in [0.1, 0.9] plus a 3x subdivided icosphere
             (1280 triangles, radius 0.3); 64^3 grid, 7 levels; one
             directional light from the upper hemisphere; 512^2 shadow map;
             640x360 G-buffer.
  large    - 4096 boxes (12 triangles each) and 64 floor-to-ceiling cylinder
             columns (3328 side triangles each) = 262,144 triangles, sizes
             log-uniform in 0.01-0.2 of the scene extent, albedo in [0,1]^3
             per instance; 256^3 grid, 9 levels; one directional light plus
             4 point lights; 2048^2 shadow map; 1920x1080 G-buffer.
  obj      - an OBJ mesh (parse_obj / obj_scene: the reference's
             resources/*.obj loaded as its tinyobjloader does) inside the
             Cornell walls.

Matrices follow glm's formulas (column-major float32, flattened
column by column as GLSL stores them).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

DEG = np.pi / 180.0


# --------------------------------------------------------------- matrices
def _normalize(v):
    v = np.asarray(v, dtype=np.float64)
    return v / np.linalg.norm(v)


def look_at(eye, center, up) -> np.ndarray:
    """glm::lookAt (right handed) as a 4x4 row-major numpy matrix."""
    eye, center, up = (np.asarray(a, dtype=np.float64) for a in (eye, center, up))
    f = _normalize(center - eye)
    s = _normalize(np.cross(f, up))
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3] = s
    m[1, :3] = u
    m[2, :3] = -f
    m[0, 3] = -s @ eye
    m[1, 3] = -u @ eye
    m[2, 3] = f @ eye
    return m


def ortho(l, r, b, t, n, f) -> np.ndarray:
    m = np.eye(4)
    m[0, 0] = 2 / (r - l)
    m[1, 1] = 2 / (t - b)
    m[2, 2] = -2 / (f - n)
    m[0, 3] = -(r + l) / (r - l)
    m[1, 3] = -(t + b) / (t - b)
    m[2, 3] = -(f + n) / (f - n)
    return m


def perspective(fovy, aspect, zn, zf) -> np.ndarray:
    th = np.tan(fovy / 2)
    m = np.zeros((4, 4))
    m[0, 0] = 1 / (aspect * th)
    m[1, 1] = 1 / th
    m[2, 2] = -(zf + zn) / (zf - zn)
    m[3, 2] = -1
    m[2, 3] = -(2 * zf * zn) / (zf - zn)
    return m


def colmajor(m: np.ndarray) -> np.ndarray:
    """4x4 matrix -> 16 float32 in GLSL (column-major) order."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.float64).T.reshape(16)).astype(np.float32)


# ------------------------------------------------------------------ scene
@dataclass
class Scene:
    name: str
    positions: np.ndarray  # (T, 9) float32
    normals: np.ndarray  # (T, 9) float32
    albedo: np.ndarray  # (T, 3) float32
    lights: list  # dicts: position, direction, color, range, intensity, shadow_caster, type
    dim: int
    levels: int
    vmax: float  # volume is [-vmax, vmax]^3 centred at the origin
    shadow_size: tuple
    ls: np.ndarray  # (16,) float32 column-major light projection * view
    ls_inverse: np.ndarray
    light_pos: np.ndarray  # (3,)
    light_int: np.ndarray  # (3,)
    eye: np.ndarray
    view_proj: np.ndarray  # (16,)
    inv_view_proj: np.ndarray
    gbuffer_size: tuple
    cone: dict = field(default_factory=dict)  # trace settings (radians)
    # 'pv' of the perspective warp: perspective(fov, aspect, 1, 20) * view
    # (src/Application.cpp:202), column-major
    pv: np.ndarray | None = None

    @property
    def ntri(self) -> int:
        return int(self.positions.shape[0])


def _quad(p0, p1, p2, p3, n):
    """Two CCW triangles (p0,p1,p2) and (p0,p2,p3) with a flat normal."""
    tris = np.array([[p0, p1, p2], [p0, p2, p3]], dtype=np.float64)
    nrm = np.broadcast_to(np.asarray(n, dtype=np.float64), (2, 3, 3))
    return tris, nrm


def icosphere(subdiv: int) -> np.ndarray:
    """Unit icosphere triangles (F, 3, 3) after `subdiv` 4:1 subdivisions."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11],
                  [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    tris = v[f]
    for _ in range(subdiv):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab, bc, ca = a + b, b + c, c + a
        ab /= np.linalg.norm(ab, axis=1, keepdims=True)
        bc /= np.linalg.norm(bc, axis=1, keepdims=True)
        ca /= np.linalg.norm(ca, axis=1, keepdims=True)
        tris = np.stack([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1), np.stack([ca, bc, c], 1),
                         np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3, 3)
    return tris


def _box(rng, size, center, yaw):
    """12 triangles of an axis-aligned box rotated by `yaw` about +y."""
    hx, hy, hz = np.asarray(size) / 2
    c = np.array([[-hx, -hy, -hz], [hx, -hy, -hz], [hx, hy, -hz], [-hx, hy, -hz],
                  [-hx, -hy, hz], [hx, -hy, hz], [hx, hy, hz], [-hx, hy, hz]])
    faces = [((0, 3, 2, 1), (0, 0, -1)), ((4, 5, 6, 7), (0, 0, 1)), ((0, 4, 7, 3), (-1, 0, 0)),
             ((1, 2, 6, 5), (1, 0, 0)), ((0, 1, 5, 4), (0, -1, 0)), ((3, 7, 6, 2), (0, 1, 0))]
    cs, sn = np.cos(yaw), np.sin(yaw)
    R = np.array([[cs, 0, sn], [0, 1, 0], [-sn, 0, cs]])
    tris, nrms = [], []
    for (i0, i1, i2, i3), n in faces:
        t, nn = _quad(c[i0], c[i1], c[i2], c[i3], n)
        tris.append(t)
        nrms.append(nn)
    tris = np.concatenate(tris) @ R.T + center
    nrms = np.concatenate(nrms) @ R.T
    return tris, nrms


# Corner indices and normals of the 12 triangles _box emits, in its order.
_BOX_TRI = np.array([[0, 3, 2], [0, 2, 1], [4, 5, 6], [4, 6, 7], [0, 4, 7], [0, 7, 3], [1, 2, 6], [1, 6, 5],
                     [0, 1, 5], [0, 5, 4], [3, 7, 6], [3, 6, 2]])
_BOX_NRM = np.repeat(np.array([(0, 0, -1), (0, 0, 1), (-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0)], float), 2, 0)
_BOX_CORNER = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                        [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float) * 0.5


def _boxes(size, center, yaw):
    """_box for many boxes at once: (B*12, 3, 3) triangles and normals."""
    cs, sn = np.cos(yaw), np.sin(yaw)
    R = np.zeros((len(yaw), 3, 3))
    R[:, 0, 0], R[:, 0, 2], R[:, 1, 1], R[:, 2, 0], R[:, 2, 2] = cs, sn, 1.0, -sn, cs
    local = _BOX_CORNER[_BOX_TRI][None] * size[:, None, None, :]          # (B, 12, 3, 3)
    tris = np.einsum("bij,btkj->btki", R, local) + center[:, None, None, :]
    nrms = np.einsum("bij,tj->bti", R, _BOX_NRM)[:, :, None, :].repeat(3, 2)
    return tris.reshape(-1, 3, 3), nrms.reshape(-1, 3, 3)


def _cylinder(radius, y0, y1, cx, cz, segments):
    a = np.arange(segments + 1) * (2 * np.pi / segments)
    x, z = np.cos(a), np.sin(a)
    b = np.stack([cx + radius * x, np.full_like(x, y0), cz + radius * z], 1)
    t = np.stack([cx + radius * x, np.full_like(x, y1), cz + radius * z], 1)
    n = np.stack([x, np.zeros_like(x), z], 1)
    k0, k1 = slice(0, segments), slice(1, segments + 1)
    tri1 = np.stack([b[k0], t[k1], b[k1]], 1)
    nrm1 = np.stack([n[k0], n[k1], n[k1]], 1)
    tri2 = np.stack([b[k0], t[k0], t[k1]], 1)
    nrm2 = np.stack([n[k0], n[k0], n[k1]], 1)
    tris = np.stack([tri1, tri2], 1).reshape(-1, 3, 3)
    nrms = np.stack([nrm1, nrm2], 1).reshape(-1, 3, 3)
    return tris, nrms


def _directional_light(rng, vmax):
    """Directional light from a random upper-hemisphere direction, placed
    outside the volume with an ortho frustum covering its bounding sphere."""
    y = rng.uniform(0.3, 0.95)
    phi = rng.uniform(0, 2 * np.pi)
    u = np.array([np.sqrt(1 - y * y) * np.cos(phi), y, np.sqrt(1 - y * y) * np.sin(phi)])
    direction = -u
    bound = vmax * np.sqrt(3.0)
    pos = u * (3.0 * vmax)
    ls = ortho(-bound, bound, -bound, bound, 0.0, 6.0 * vmax) @ look_at(pos, pos + direction, (0, 1, 0))
    return dict(position=pos, direction=direction, color=np.ones(3), range=5.0, intensity=1.0, shadow_caster=1,
                type=1), ls


def _finish(name, tris, nrms, alb, lights, ls, dim, levels, vmax, shadow_size, eye, target, fovy, gsize, cone):
    W, H = gsize
    vpm = perspective(fovy, W / H, 0.1, 20.0) @ look_at(eye, target, (0, 1, 0))
    main = lights[0]
    return Scene(
        name=name,
        positions=np.ascontiguousarray(tris.reshape(-1, 9), dtype=np.float32),
        normals=np.ascontiguousarray(nrms.reshape(-1, 9), dtype=np.float32),
        albedo=np.ascontiguousarray(alb, dtype=np.float32),
        lights=lights, dim=dim, levels=levels, vmax=vmax, shadow_size=shadow_size,
        ls=colmajor(ls), ls_inverse=colmajor(np.linalg.inv(ls)),
        light_pos=np.asarray(main["position"], dtype=np.float32),
        light_int=np.asarray(main["color"], dtype=np.float32),
        eye=np.asarray(eye, dtype=np.float32), view_proj=colmajor(vpm), inv_view_proj=colmajor(np.linalg.inv(vpm)),
        gbuffer_size=gsize, cone=cone,
        pv=colmajor(perspective(fovy, W / H, 1.0, 20.0) @ look_at(eye, target, (0, 1, 0))))


# The benchmark frames' cones (steps, aperture, bias, initial height, LOD offset): 6 diffuse
# cones of 60 degrees and one specular cone of 10 degrees.
FRAME_CONES = dict(diffuse=(16, 60 * DEG, 1.0, 1.0, 0.5), specular=(32, 10 * DEG, 1.7, 0.5, 0.1))


def cornell(seed: int = 0, dim: int = 64, shadow: int = 512, gbuffer=(640, 360)) -> Scene:
    rng = np.random.default_rng(seed)
    w = 0.95
    walls = [
        ((-w, -w, -w), (-w, -w, w), (w, -w, w), (w, -w, -w), (0, 1, 0)),    # floor
        ((-w, -w, -w), (w, -w, -w), (w, w, -w), (-w, w, -w), (0, 0, 1)),    # back
        ((-w, -w, w), (-w, w, w), (w, w, w), (w, -w, w), (0, 0, -1)),       # front
        ((-w, -w, -w), (-w, w, -w), (-w, w, w), (-w, -w, w), (1, 0, 0)),    # left
        ((w, -w, -w), (w, -w, w), (w, w, w), (w, w, -w), (-1, 0, 0)),       # right
    ]
    tris, nrms, alb = [], [], []
    for p0, p1, p2, p3, n in walls:
        t, nn = _quad(np.array(p0), np.array(p1), np.array(p2), np.array(p3), n)
        tris.append(t)
        nrms.append(nn)
        alb.append(np.repeat(rng.uniform(0.1, 0.9, size=(1, 3)), 2, 0))
    sph = icosphere(3)
    c = rng.uniform(-0.6, 0.6, size=3)
    tris.append(sph * 0.3 + c)
    nrms.append(sph.copy())
    alb.append(np.repeat(rng.uniform(0.1, 0.9, size=(1, 3)), sph.shape[0], 0))
    light, ls = _directional_light(rng, 1.0)
    levels = int(np.log2(dim)) + 1
    return _finish("cornell", np.concatenate(tris), np.concatenate(nrms), np.concatenate(alb), [light], ls, dim,
                   levels, 1.0, (shadow, shadow), np.array([0.0, 1.6, 2.6]), np.array([0.0, -0.4, 0.0]), 50 * DEG,
                   tuple(gbuffer), FRAME_CONES)


def large(seed: int = 0, dim: int = 256, shadow: int = 2048, gbuffer=(1920, 1080), n_boxes: int = 4096,
          n_cyl: int = 64, cyl_segments: int = 1664) -> Scene:
    rng = np.random.default_rng(seed)
    extent = 2.0
    lo, hi = np.log(0.01 * extent), np.log(0.2 * extent)
    tris, nrms, alb = [], [], []
    for _ in range(n_boxes):
        size = np.exp(rng.uniform(lo, hi, size=3))
        center = rng.uniform(-0.9, 0.9, size=3)
        yaw = rng.uniform(0, 2 * np.pi)
        t, n = _box(rng, size, center, yaw)
        tris.append(t)
        nrms.append(n)
        alb.append(np.repeat(rng.uniform(0, 1, size=(1, 3)), 12, 0))
    for _ in range(n_cyl):
        radius = 0.5 * np.exp(rng.uniform(lo, hi))
        cx, cz = rng.uniform(-0.9, 0.9, size=2)
        t, n = _cylinder(radius, -0.95, 0.95, cx, cz, cyl_segments)
        tris.append(t)
        nrms.append(n)
        alb.append(np.repeat(rng.uniform(0, 1, size=(1, 3)), t.shape[0], 0))
    light, ls = _directional_light(rng, 1.0)
    lights = [light]
    for _ in range(4):
        lights.append(dict(position=rng.uniform(-0.9, 0.9, size=3), direction=np.array([0.0, -1.0, 0.0]),
                           color=rng.uniform(0.5, 1.0, size=3), range=float(rng.uniform(0.3, 0.8)), intensity=1.0,
                           shadow_caster=0, type=0))
    levels = int(np.log2(dim)) + 1
    return _finish("large", np.concatenate(tris), np.concatenate(nrms), np.concatenate(alb), lights, ls, dim, levels,
                   1.0, (shadow, shadow), np.array([0.0, 0.5, 2.8]), np.array([0.0, 0.0, 0.0]), 55 * DEG,
                   tuple(gbuffer), FRAME_CONES)


def tiny(seed: int = 0, dim: int = 16, shadow: int = 64, gbuffer=(48, 32), n_boxes: int = 6) -> Scene:
    """A few boxes in a 16^3 grid: small enough for pure-CPU oracle tests."""
    rng = np.random.default_rng(seed)
    tris, nrms, alb = [], [], []
    for _ in range(n_boxes):
        size = rng.uniform(0.2, 0.8, size=3)
        center = rng.uniform(-0.6, 0.6, size=3)
        t, n = _box(rng, size, center, rng.uniform(0, 2 * np.pi))
        tris.append(t)
        nrms.append(n)
        alb.append(np.repeat(rng.uniform(0, 1, size=(1, 3)), 12, 0))
    light, ls = _directional_light(rng, 1.0)
    lights = [light, dict(position=np.array([0.2, 0.5, 0.1]), direction=np.array([0.0, -1.0, 0.0]),
                          color=np.array([1.0, 0.8, 0.6]), range=1.5, intensity=1.0, shadow_caster=0, type=0)]
    levels = int(np.log2(dim)) + 1
    return _finish("tiny", np.concatenate(tris), np.concatenate(nrms), np.concatenate(alb), lights, ls, dim, levels,
                   1.0, (shadow, shadow), np.array([0.3, 0.9, 2.4]), np.array([0.0, 0.0, 0.0]), 50 * DEG,
                   tuple(gbuffer), FRAME_CONES)


def stacked_slivers(copies: int = 1600, seed: int = 0, dim: int = 64, shadow: int = 64,
                    gbuffer=(64, 36)) -> Scene:
    """`copies` coincident long thin triangles (a sliver along x inside one
    row of voxels, each copy with its own albedo): the tessellation
    voxeliser puts ~48 points per copy into each voxel of the row, so with
    more than ~1,400 copies a voxel receives more than 65,536 points and its
    sums pass 2^32."""
    rng = np.random.default_rng(seed)
    tri = np.array([[-0.9, 0.010, 0.013], [0.9, 0.010, 0.013], [0.9, 0.012, 0.0135]], dtype=np.float64)
    n = np.cross(tri[1] - tri[0], tri[2] - tri[0])
    n /= np.linalg.norm(n)
    tris = np.repeat(tri[None], copies, 0)
    nrms = np.repeat(np.repeat(n[None, None], 3, 1), copies, 0)
    alb = rng.uniform(0, 1, size=(copies, 3))
    light, ls = _directional_light(rng, 1.0)
    levels = int(np.log2(dim)) + 1
    return _finish("slivers", tris, nrms, alb, [light], ls, dim, levels, 1.0, (shadow, shadow),
                   np.array([0.0, 0.5, 2.5]), np.zeros(3), 50 * DEG, tuple(gbuffer), FRAME_CONES)


# Batched scene family: per scene a triangle count log-uniform in [1k, 200k]
# (rotated boxes of log-uniform size), a grid from {64, 128, 256}^3, a 16:9
# G-buffer from 320x180 to 1920x1080 and 1-4 lights (one directional shadow
# caster plus point lights).
BATCH_DIMS = (64, 128, 256)
BATCH_GBUFFERS = tuple((320 * k, 180 * k) for k in range(1, 7))


def batch_scene(seed: int = 0, index: int = 0, shadow: int = 1024) -> Scene:
    rng = np.random.default_rng((seed, index))
    ntri = int(np.exp(rng.uniform(np.log(1000), np.log(200000))))
    n_boxes = max(1, ntri // 12)
    dim = int(rng.choice(BATCH_DIMS))
    gsize = BATCH_GBUFFERS[int(rng.integers(len(BATCH_GBUFFERS)))]
    extent = 2.0
    # Smaller boxes in denser scenes keep the covered area comparable.
    hi = np.log(0.2 * extent * min(1.0, (2000.0 / n_boxes) ** 0.5) + 0.02)
    lo = np.log(0.01 * extent)
    size = np.exp(rng.uniform(lo, max(hi, lo + 0.1), size=(n_boxes, 3)))
    center = rng.uniform(-0.9, 0.9, size=(n_boxes, 3))
    yaw = rng.uniform(0, 2 * np.pi, size=n_boxes)
    tris, nrms = _boxes(size, center, yaw)
    alb = np.repeat(rng.uniform(0, 1, size=(n_boxes, 3)), 12, 0)
    light, ls = _directional_light(rng, 1.0)
    lights = [light]
    for _ in range(int(rng.integers(0, 4))):
        lights.append(dict(position=rng.uniform(-0.9, 0.9, size=3), direction=np.array([0.0, -1.0, 0.0]),
                           color=rng.uniform(0.5, 1.0, size=3), range=float(rng.uniform(0.3, 0.8)), intensity=1.0,
                           shadow_caster=0, type=0))
    phi = rng.uniform(0, 2 * np.pi)
    eye = np.array([2.8 * np.sin(phi), rng.uniform(0.2, 1.0), 2.8 * np.cos(phi)])
    levels = int(np.log2(dim)) + 1
    return _finish(f"batch{index}", tris, nrms, alb, lights, ls, dim, levels, 1.0, (shadow, shadow), eye,
                   np.zeros(3), 55 * DEG, gsize, FRAME_CONES)


def _cylinders(radius, y0, y1, cx, cz, segments):
    """_cylinder for many columns at once (same triangle order)."""
    a = np.arange(segments + 1) * (2 * np.pi / segments)
    x, z = np.cos(a), np.sin(a)
    C = len(radius)
    bx = cx[:, None] + radius[:, None] * x[None]
    bz = cz[:, None] + radius[:, None] * z[None]
    b = np.stack([bx, np.full_like(bx, y0), bz], -1)
    t = np.stack([bx, np.full_like(bx, y1), bz], -1)
    n = np.broadcast_to(np.stack([x, np.zeros_like(x), z], -1), (C, segments + 1, 3))
    k0, k1 = slice(0, segments), slice(1, segments + 1)
    tri1 = np.stack([b[:, k0], t[:, k1], b[:, k1]], 2)
    nrm1 = np.stack([n[:, k0], n[:, k1], n[:, k1]], 2)
    tri2 = np.stack([b[:, k0], t[:, k0], t[:, k1]], 2)
    nrm2 = np.stack([n[:, k0], n[:, k0], n[:, k1]], 2)
    return np.stack([tri1, tri2], 2).reshape(-1, 3, 3), np.stack([nrm1, nrm2], 2).reshape(-1, 3, 3)


def large_family(seed: int = 0, dim: int = 256, shadow: int = 2048, gbuffer=(1920, 1080), n_boxes: int = 4096,
                 n_cyl: int = 64, cyl_segments: int = 1664, orbit: bool = True) -> Scene:
    """The large plain frame's family, generated with vectorised draws: the
    same box / column / light distributions as large() (which it does not
    reproduce draw for draw), and with `orbit` a camera at a random azimuth
    and height around the volume.  Used for the learned path's training and
    held-out scenes."""
    rng = np.random.default_rng((seed, 7))
    extent = 2.0
    lo, hi = np.log(0.01 * extent), np.log(0.2 * extent)
    size = np.exp(rng.uniform(lo, hi, size=(n_boxes, 3)))
    center = rng.uniform(-0.9, 0.9, size=(n_boxes, 3))
    yaw = rng.uniform(0, 2 * np.pi, size=n_boxes)
    bt, bn = _boxes(size, center, yaw)
    balb = np.repeat(rng.uniform(0, 1, size=(n_boxes, 3)), 12, 0)
    radius = 0.5 * np.exp(rng.uniform(lo, hi, size=n_cyl))
    cxz = rng.uniform(-0.9, 0.9, size=(n_cyl, 2))
    ct, cn = _cylinders(radius, -0.95, 0.95, cxz[:, 0], cxz[:, 1], cyl_segments)
    calb = np.repeat(rng.uniform(0, 1, size=(n_cyl, 3)), 2 * cyl_segments, 0)
    light, ls = _directional_light(rng, 1.0)
    lights = [light]
    for _ in range(4):
        lights.append(dict(position=rng.uniform(-0.9, 0.9, size=3), direction=np.array([0.0, -1.0, 0.0]),
                           color=rng.uniform(0.5, 1.0, size=3), range=float(rng.uniform(0.3, 0.8)), intensity=1.0,
                           shadow_caster=0, type=0))
    if orbit:
        phi = rng.uniform(0, 2 * np.pi)
        eye = np.array([2.8 * np.sin(phi), rng.uniform(0.2, 1.0), 2.8 * np.cos(phi)])
    else:
        eye = np.array([0.0, 0.5, 2.8])
    levels = int(np.log2(dim)) + 1
    return _finish(f"family{seed}", np.concatenate([bt, ct]), np.concatenate([bn, cn]), np.concatenate([balb, calb]),
                   lights, ls, dim, levels, 1.0, (shadow, shadow), eye, np.zeros(3), 55 * DEG, tuple(gbuffer),
                   FRAME_CONES)


# Dynamic family: rigid actors (cylinders of 1k-4k segments, 2k-8k triangles)
# with random linear and angular velocities in a static environment of the
# large frame's family (4,096 boxes and 45 columns: 198,912 triangles).
@dataclass
class Actors:
    first: np.ndarray      # (A,) first triangle of each actor in the scene's arrays
    count: np.ndarray      # (A,) triangles per actor
    p0: np.ndarray         # (A, 3) initial positions
    vel: np.ndarray        # (A, 3) linear velocities (units / s)
    axis: np.ndarray       # (A, 3) unit rotation axes
    omega: np.ndarray      # (A,) angular speeds (rad / s)

    def model(self, k: int, t: float) -> np.ndarray:
        """Row-major 4x4 model of actor k at time t: translate(p(t)) * rotate(axis, omega t);
        positions bounce inside [-0.8, 0.8]^3."""
        p = self.p0[k] + self.vel[k] * t
        p = 0.8 - np.abs(np.mod(p + 0.8, 3.2) - 1.6)  # triangle wave in [-0.8, 0.8]
        a = self.axis[k]
        ang = self.omega[k] * t
        c, s_ = np.cos(ang), np.sin(ang)
        K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
        R = np.eye(3) + s_ * K + (1 - c) * (K @ K)
        M = np.eye(4)
        M[:3, :3] = R
        M[:3, 3] = p
        return M

    def models(self, t: float) -> list:
        return [(int(self.first[k]), int(self.count[k]), self.model(k, t)) for k in range(len(self.first))]


def dynamic_scene(seed: int = 0, n_actors: int = 64, dim: int = 256, shadow: int = 2048, gbuffer=(1280, 720),
                  static_boxes: int = 4096, static_cyl: int = 45) -> tuple:
    """(scene, actors): the scene's triangle arrays hold the static environment
    followed by every actor's mesh in its local frame (centred at the
    origin); actors.model(k, t) places actor k at time t."""
    env = large_family(seed, dim=dim, shadow=shadow, gbuffer=gbuffer, n_boxes=static_boxes, n_cyl=static_cyl,
                       orbit=False)
    rng = np.random.default_rng((seed, 11))
    tris, nrms, albs = [env.positions.reshape(-1, 3, 3)], [env.normals.reshape(-1, 3, 3)], [env.albedo]
    first, count = [], []
    t0 = env.ntri
    for _ in range(n_actors):
        seg = int(rng.integers(1000, 4001))
        r = float(rng.uniform(0.03, 0.1))
        h = float(rng.uniform(0.1, 0.4))
        t, n = _cylinders(np.array([r]), -h / 2, h / 2, np.zeros(1), np.zeros(1), seg)
        tris.append(t)
        nrms.append(n)
        albs.append(np.repeat(rng.uniform(0, 1, size=(1, 3)), t.shape[0], 0))
        first.append(t0)
        count.append(t.shape[0])
        t0 += t.shape[0]
    A = len(first)
    axis = rng.normal(size=(A, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    actors = Actors(first=np.array(first, np.int64), count=np.array(count, np.int64),
                    p0=rng.uniform(-0.8, 0.8, size=(A, 3)), vel=rng.uniform(-0.4, 0.4, size=(A, 3)), axis=axis,
                    omega=rng.uniform(-2.0, 2.0, size=A))
    sc = _finish(f"dynamic{seed}", np.concatenate(tris).astype(np.float64), np.concatenate(nrms).astype(np.float64),
                 np.concatenate(albs), env.lights, np.eye(4), dim, env.levels, 1.0, env.shadow_size,
                 np.array([0.0, 0.5, 2.8]), np.zeros(3), 55 * DEG, tuple(gbuffer), FRAME_CONES)
    # keep the environment's light-space matrices
    sc.ls, sc.ls_inverse = env.ls, env.ls_inverse
    return sc, actors


def viewpoint(sc: Scene, k: int, n: int = 8, radius: float = 2.8) -> Scene:
    """The scene seen from the k-th of n cameras on a circle around the volume."""
    import copy

    v = copy.copy(sc)
    phi = 2 * np.pi * k / n
    eye = np.array([radius * np.sin(phi), 0.5, radius * np.cos(phi)])
    W, H = sc.gbuffer_size
    vpm = perspective(55 * DEG, W / H, 0.1, 20.0) @ look_at(eye, np.zeros(3), (0, 1, 0))
    v.eye = eye.astype(np.float32)
    v.view_proj = colmajor(vpm)
    v.inv_view_proj = colmajor(np.linalg.inv(vpm))
    v.pv = colmajor(perspective(55 * DEG, W / H, 1.0, 20.0) @ look_at(eye, np.zeros(3), (0, 1, 0)))
    return v


# ------------------------------------------------------------ OBJ meshes
def parse_obj(text: str):
    """Triangles of a Wavefront OBJ text as the reference's loader reads
    them (tinyobjloader with triangulation, src/Graphics/Mesh.cpp:41-190):
    `v` and `vn` records, faces of `v`, `v/vt`, `v//vn` or `v/vt/vn` indices
    (1-based, negative = relative to the end), polygons split into a fan
    (0, i, i+1) around their first vertex, and a zero normal for a face
    corner without one (the loader's zero-initialised vertex).  Returns
    positions (T, 3, 3), normals (T, 3, 3) and the face's object index
    (T,) counting `o`/`g` records."""
    vs, vns, tris, nrms, groups = [], [], [], [], []
    group = 0
    seen_face = False
    for line in text.splitlines():
        parts = line.split()
        if not parts or parts[0].startswith("#"):
            continue
        tag = parts[0]
        if tag == "v":
            vs.append([float(x) for x in parts[1:4]])
        elif tag == "vn":
            vns.append([float(x) for x in parts[1:4]])
        elif tag in ("o", "g"):
            if seen_face:
                group += 1
                seen_face = False
        elif tag == "f":
            corners = []
            for c in parts[1:]:
                f = c.split("/")
                vi = int(f[0])
                vi = vi - 1 if vi > 0 else len(vs) + vi
                ni = None
                if len(f) >= 3 and f[2]:
                    ni = int(f[2])
                    ni = ni - 1 if ni > 0 else len(vns) + ni
                corners.append((vi, ni))
            for i in range(1, len(corners) - 1):
                tri = (corners[0], corners[i], corners[i + 1])
                tris.append([vs[k] for k, _ in tri])
                nrms.append([vns[n] if n is not None else [0.0, 0.0, 0.0] for _, n in tri])
                groups.append(group)
            seen_face = True
    return (np.asarray(tris, dtype=np.float64).reshape(-1, 3, 3), np.asarray(nrms, dtype=np.float64).reshape(-1, 3, 3),
            np.asarray(groups, dtype=np.int64))


def load_obj(path: str):
    with open(path) as f:
        return parse_obj(f.read())


def obj_scene(text: str, seed: int = 0, dim: int = 64, shadow: int = 512, gbuffer=(640, 360), size: float = 0.7,
              walls: bool = True) -> Scene:
    """A parity scene around an OBJ mesh (the reference's resources/*.obj):
    the mesh scaled uniformly so its bounding box spans `size` of the volume
    [-1, 1]^3 and centred, inside the Cornell walls; one albedo per OBJ
    object; the Cornell box's camera and light."""
    rng = np.random.default_rng(seed)
    tris, nrms, groups = parse_obj(text)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    scale = 2.0 * size / max(float((hi - lo).max()), 1e-12)
    tris = (tris - 0.5 * (lo + hi)) * scale
    alb_groups = rng.uniform(0.1, 0.9, size=(int(groups.max()) + 1 if len(groups) else 1, 3))
    alb = alb_groups[groups]
    parts_t, parts_n, parts_a = [tris], [nrms], [alb]
    if walls:
        base = cornell(seed=seed, dim=dim)
        k = 10  # the five wall quads
        parts_t.insert(0, base.positions[:k].reshape(-1, 3, 3).astype(np.float64))
        parts_n.insert(0, base.normals[:k].reshape(-1, 3, 3).astype(np.float64))
        parts_a.insert(0, base.albedo[:k].astype(np.float64))
    light, ls = _directional_light(rng, 1.0)
    levels = int(np.log2(dim)) + 1
    return _finish("obj", np.concatenate(parts_t), np.concatenate(parts_n), np.concatenate(parts_a), [light], ls, dim,
                   levels, 1.0, (shadow, shadow), np.array([0.0, 1.6, 2.6]), np.array([0.0, -0.4, 0.0]), 50 * DEG,
                   tuple(gbuffer), FRAME_CONES)


def obj_text(tris: np.ndarray, normals: np.ndarray | None = None, quads: bool = False) -> str:
    """OBJ text of a triangle soup (F, 3, 3), with `vn` records when normals
    are given; with `quads` consecutive triangle pairs (p0,p1,p2), (p0,p2,p3)
    are written as one quad face.  Used to build OBJ inputs for the loader."""
    lines = ["# generated"]
    v = tris.reshape(-1, 3)
    lines += [f"v {a:.9g} {b:.9g} {c:.9g}" for a, b, c in v]
    if normals is not None:
        lines += [f"vn {a:.9g} {b:.9g} {c:.9g}" for a, b, c in normals.reshape(-1, 3)]
    fmt = (lambda i: f"{i}//{i}") if normals is not None else (lambda i: f"{i}")
    F = tris.shape[0]
    if quads:
        for t in range(0, F - 1, 2):
            i = 3 * t + 1
            lines.append("f " + " ".join(fmt(k) for k in (i, i + 1, i + 2, i + 5)))
    else:
        for t in range(F):
            i = 3 * t + 1
            lines.append("f " + " ".join(fmt(k) for k in (i, i + 1, i + 2)))
    return "\n".join(lines) + "\n"


SCENES = {"cornell": cornell, "large": large, "tiny": tiny}


def make(name: str, seed: int = 0, **kw) -> Scene:
    return SCENES[name](seed=seed, **kw)
