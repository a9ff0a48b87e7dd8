"""numpy binding of the CPU oracle (liboracle.so, built from vct_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  The oracle is the correctness reference of the CUDA
library and the timed CPU baseline.  Only tests/, the smoke check and the
benchmark's CPU-baseline leg use it; the product never imports it.

Parity status: unpinned by the reference.  The reference (sfreed141/vct)
ships no tests, fixtures or golden outputs and its OpenGL/GLSL program
cannot run here (no graphics stack), so the oracle is pinned instead by
hand-computed known answers in tests/golden (see tests/golden/make_golden.py).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_lib = None


class orc_volume(C.Structure):
    _fields_ = [("dim", C.c_int32), ("vmin", C.c_float * 3), ("vmax", C.c_float * 3), ("vcenter", C.c_float * 3)]


class orc_light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("_p0", C.c_float), ("direction", C.c_float * 3), ("_p1", C.c_float),
                ("color", C.c_float * 3), ("range", C.c_float), ("intensity", C.c_float), ("enabled", C.c_uint32),
                ("selected", C.c_uint32), ("shadow_caster", C.c_uint32), ("type", C.c_uint32),
                ("_p2", C.c_uint32 * 3)]


class orc_cone(C.Structure):
    _fields_ = [("steps", C.c_int32), ("angle", C.c_float), ("bias", C.c_float), ("h0", C.c_float),
                ("lod_offset", C.c_float)]


class orc_trace_params(C.Structure):
    _fields_ = [("diffuse", orc_cone), ("specular", orc_cone), ("enable_indirect", C.c_int32),
                ("enable_reflections", C.c_int32), ("draw_occlusion", C.c_int32), ("enable_postprocess", C.c_int32),
                ("ambient_scale", C.c_float), ("reflect_scale", C.c_float), ("max_distance", C.c_float),
                ("ref_tbn_quirk", C.c_int32)]


class orc_warp(C.Structure):
    _fields_ = [("mode", C.c_int32), ("map", C.c_void_p), ("eye_tc", C.c_float * 3), ("pv", C.c_float * 16),
                ("vmin", C.c_float * 3), ("vcenter", C.c_float * 3), ("ext", C.c_float * 3)]


class orc_shade_params(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("cooktorrance", "enable_diffuse", "enable_specular", "enable_indirect",
                                         "enable_reflections", "draw_occlusion", "enable_postprocess")] + \
               [(k, C.c_float) for k in ("roughness", "metallic", "shininess", "ambient_scale", "reflect_scale")]


class orc_stats(C.Structure):
    _fields_ = [("total_voxel_fragments", C.c_uint32), ("unique_voxels", C.c_uint32),
                ("max_fragments_per_voxel", C.c_uint32), ("error_flags", C.c_uint32)]


def build() -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _p(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)


def _f(v, n):
    return (C.c_float * n)(*np.asarray(v, dtype=np.float32).reshape(n).tolist())


def volume(scene, dim: int | None = None) -> orc_volume:
    v = orc_volume()
    v.dim = int(dim or scene.dim)
    v.vmin = _f([-scene.vmax] * 3, 3)
    v.vmax = _f([scene.vmax] * 3, 3)
    v.vcenter = _f([0, 0, 0], 3)
    return v


def lights(scene):
    arr = (orc_light * max(1, len(scene.lights)))()
    for i, d in enumerate(scene.lights):
        li = arr[i]
        li.position = _f(d["position"], 3)
        li.direction = _f(d["direction"], 3)
        li.color = _f(d["color"], 3)
        li.range = float(d["range"])
        li.intensity = float(d["intensity"])
        li.enabled = int(d.get("enabled", 1))
        li.shadow_caster = int(d.get("shadow_caster", 0))
        li.type = int(d["type"])
    return arr, len(scene.lights)


def trace_params(scene, **over) -> orc_trace_params:
    t = orc_trace_params()
    for key in ("diffuse", "specular"):
        steps, ang, bias, h0, lod = scene.cone[key]
        setattr(t, key, orc_cone(int(steps), float(ang), float(bias), float(h0), float(lod)))
    t.enable_indirect = 1
    t.enable_reflections = 1
    t.draw_occlusion = 1
    t.enable_postprocess = 1
    t.ambient_scale = 1.0
    t.reflect_scale = 1.0
    t.max_distance = float(np.sqrt(3.0))
    t.ref_tbn_quirk = 0
    for k, v in over.items():
        setattr(t, k, v)
    return t


def f32_to_f16(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(x.shape, dtype=np.uint16)
    load().orc_f32_to_f16_array(_p(x), _p(out), C.c_int64(x.size))
    return out


def voxel_mvp(scene) -> np.ndarray:
    out = np.zeros(48, dtype=np.float32)
    v = volume(scene)
    load().orc_voxel_mvp(C.byref(v), _p(out))
    return out


def warp(scene, mode: int = 0, warpmap: np.ndarray | None = None):
    """orc_warp of a scene: mode 1 warps about the eye (warpVoxels), mode 2
    reads `warpmap` (32^3 x 4 uint16, from warpmap()), mode 3 projects with
    the scene's `pv` (voxelizeTesselationWarp).  The struct keeps a reference
    to the map."""
    w = orc_warp()
    w.mode = int(mode)
    if getattr(scene, "pv", None) is not None:
        w.pv = _f(scene.pv, 16)
    w.vmin = _f([-scene.vmax] * 3, 3)
    w.vcenter = _f([0, 0, 0], 3)
    w.ext = _f([np.float32(scene.vmax) - np.float32(-scene.vmax)] * 3, 3)
    if warpmap is not None:
        w._map = np.ascontiguousarray(warpmap, dtype=np.uint16)
        w.map = w._map.ctypes.data
    # voxelLinearPosition(eye) in fp32: ((eye - center) - min) / (max - min)
    e = np.asarray(scene.eye, dtype=np.float32)
    vmin, ext = np.float32(-scene.vmax), np.float32(2 * scene.vmax)
    w.eye_tc = _f([((e[k] - np.float32(0.0)) - vmin) / ext for k in range(3)], 3)
    return w


def warpmap(occupancy: np.ndarray, high: float = 2.0, low: float = 0.5) -> np.ndarray:
    """The 32^3 warp map (32^3 x 4 uint16) of a 32^3 occupancy grid."""
    occ = np.ascontiguousarray(np.asarray(occupancy).reshape(-1) != 0, dtype=np.uint8)
    out = np.zeros(32 ** 3 * 4, dtype=np.uint16)
    load().orc_warpmap(_p(occ), C.c_float(high), C.c_float(low), _p(out))
    return out


def warp_occupancy(scene, shadowmap: np.ndarray, nthreads: int = 1) -> np.ndarray:
    """The 32^3 occupancy voxelisation of the scene (bool per cell)."""
    count, _, _ = voxelize(scene, shadowmap, lighting=0, nthreads=nthreads, dim=32)
    return count > 0


def voxelize(scene, shadowmap: np.ndarray, lighting: int = 1, axis_override: int = -1, nthreads: int = 1,
             positions=None, normals=None, albedo=None, dim: int | None = None, warp=None):
    """Returns (count[N^3] u32, sums[6*N^3] u64, total_fragments)."""
    N = int(dim or scene.dim)
    pos = np.ascontiguousarray(scene.positions if positions is None else positions, dtype=np.float32)
    nrm = np.ascontiguousarray(scene.normals if normals is None else normals, dtype=np.float32)
    alb = np.ascontiguousarray(scene.albedo if albedo is None else albedo, dtype=np.float32)
    count = np.zeros(N ** 3, dtype=np.uint32)
    sums = np.zeros(6 * N ** 3, dtype=np.uint64)
    total = C.c_uint32(0)
    arr, n = lights(scene)
    v = volume(scene, N)
    sm = np.ascontiguousarray(shadowmap, dtype=np.float32)
    sw, sh = scene.shadow_size
    load().orc_voxelize(C.byref(v), _p(pos), _p(nrm), _p(alb), C.c_int64(pos.shape[0]), arr, n, lighting,
                        axis_override, _p(sm), sw, sh, _f(scene.ls, 16), _p(count), _p(sums), C.byref(total),
                        nthreads, C.byref(warp) if warp is not None else None)
    return count, sums, int(total.value)


def tess_levels(scene, tri, max_level: float = 64.0, dim: int | None = None):
    """Tessellation levels (inner, outer0, outer1, outer2) of one triangle
    (9 floats), or None when the control shader discards it."""
    v = volume(scene, dim)
    t = np.ascontiguousarray(tri, dtype=np.float32).reshape(9)
    out = np.zeros(4, dtype=np.int32)
    ok = load().orc_tess_levels(C.byref(v), _p(t), C.c_float(max_level), _p(out))
    return tuple(int(x) for x in out) if ok else None


def tess_coords(levels) -> np.ndarray:
    """gl_TessCoord of every point GL's triangle tessellation generates in
    point mode for (inner, outer0, outer1, outer2), (npoints, 3) float32."""
    lv = np.ascontiguousarray(levels, dtype=np.int32)
    lib = load()
    n = lib.orc_tess_point_count(_p(lv))
    out = np.zeros((n, 3), dtype=np.float32)
    lib.orc_tess_coords(_p(lv), _p(out))
    return out


def voxelize_tess(scene, max_level: float = 64.0, nthreads: int = 1, positions=None, normals=None, albedo=None,
                  dim: int | None = None, warp=None):
    """The tessellation voxeliser: (count[N^3], sums[6*N^3], total_points)."""
    N = int(dim or scene.dim)
    pos = np.ascontiguousarray(scene.positions if positions is None else positions, dtype=np.float32)
    nrm = np.ascontiguousarray(scene.normals if normals is None else normals, dtype=np.float32)
    alb = np.ascontiguousarray(scene.albedo if albedo is None else albedo, dtype=np.float32)
    count = np.zeros(N ** 3, dtype=np.uint32)
    sums = np.zeros(6 * N ** 3, dtype=np.uint64)
    total = C.c_uint64(0)
    v = volume(scene, N)
    load().orc_voxelize_tess(C.byref(v), _p(pos), _p(nrm), _p(alb), C.c_int64(pos.shape[0]), C.c_float(max_level),
                             C.byref(warp) if warp is not None else None, _p(count), _p(sums), C.byref(total),
                             nthreads)
    return count, sums, int(total.value)


def normalize(scene, count, sums, opacity=0.5, temporal=0, decay=0.8, radiance=None, nthreads=1, dim=None,
              chain_voxels=None):
    """Returns (color, normal, radiance, stats); radiance is level 0 (or the
    given array, updated in place, when the temporal filter reads it)."""
    N = int(dim or scene.dim)
    nv = N ** 3
    count = np.ascontiguousarray(count, dtype=np.uint32)
    sums = np.ascontiguousarray(sums, dtype=np.uint64)
    color = np.zeros(4 * nv, dtype=np.uint16)
    normal = np.zeros(4 * nv, dtype=np.uint16)
    rad = radiance if radiance is not None else np.zeros(4 * (chain_voxels or nv), dtype=np.uint16)
    st = orc_stats()
    v = volume(scene, N)
    load().orc_normalize(C.byref(v), C.c_float(opacity), temporal, C.c_float(decay), _p(count), _p(sums),
                         _p(color), _p(normal), _p(rad), C.byref(st), nthreads)
    stats = dict(unique_voxels=st.unique_voxels, max_fragments_per_voxel=st.max_fragments_per_voxel,
                 error_flags=st.error_flags)
    return color, normal, rad, stats


def inject(scene, shadowmap, color, normal, radiance, lighting=0, dilate=0, nthreads=1, dim=None, warp=None,
           temporal=0, decay=0.8):
    N = int(dim or scene.dim)
    v = volume(scene, N)
    sw, sh = scene.shadow_size
    sm = np.ascontiguousarray(shadowmap, dtype=np.float32)
    load().orc_inject(C.byref(v), _p(sm), sw, sh, _f(scene.ls_inverse, 16), _f(scene.light_pos, 3),
                      _f(scene.light_int, 3), lighting, dilate, _p(color), _p(normal), _p(radiance), nthreads,
                      C.byref(warp) if warp is not None else None, int(temporal), C.c_float(decay))
    return radiance


def chain_voxels(dim: int, levels: int) -> int:
    return sum((dim >> l) ** 3 for l in range(levels))


def level_offsets(dim: int, levels: int) -> list[int]:
    offs, o = [], 0
    for l in range(levels):
        offs.append(o)
        o += (dim >> l) ** 3
    return offs


def build_mips(dim: int, levels: int, chain: np.ndarray, nthreads: int = 1) -> np.ndarray:
    load().orc_build_mips(dim, levels, _p(chain), nthreads)
    return chain


def trace(scene, chain, gpos, gnrm, galb, precision=32, rows=None, row_step=1, nthreads=1, want=("irr", "spec",
                                                                                                  "color"), warp=None,
          **over):
    W, H = scene.gbuffer_size
    r0, r1 = rows if rows is not None else (0, H)
    tp = trace_params(scene, **over)
    v = volume(scene)
    irr = np.zeros((H * W * 4,), dtype=np.float32) if "irr" in want else None
    spec = np.zeros((H * W * 4,), dtype=np.float32) if "spec" in want else None
    col = np.zeros((H * W * 4,), dtype=np.float32) if "color" in want else None
    samples = C.c_uint64(0)
    load().orc_trace(C.byref(v), scene.levels, _p(chain), C.byref(tp), _p(gpos), _p(gnrm), _p(galb), W, H, r0, r1,
                     row_step, _f(scene.eye, 3), precision, _p(irr), _p(spec), _p(col), C.byref(samples), nthreads,
                     C.byref(warp) if warp is not None else None)
    return irr, spec, col, int(samples.value)


def render_shadowmap(scene, nthreads=1) -> np.ndarray:
    W, H = scene.shadow_size
    out = np.empty(W * H, dtype=np.float32)
    load().orc_render_shadowmap(_p(scene.positions), C.c_int64(scene.ntri), _f(scene.ls, 16), W, H, _p(out), nthreads)
    return out


def render_gbuffer(scene):
    W, H = scene.gbuffer_size
    gp = np.zeros(W * H * 4, dtype=np.float32)
    gn = np.zeros(W * H * 4, dtype=np.float32)
    ga = np.zeros(W * H * 4, dtype=np.float32)
    load().orc_render_gbuffer(_p(scene.positions), _p(scene.normals), _p(scene.albedo), C.c_int64(scene.ntri),
                              _f(scene.view_proj, 16), _f(scene.eye, 3), _f(scene.inv_view_proj, 16), W, H, _p(gp),
                              _p(gn), _p(ga))
    return gp, gn, ga


def f16_to_f32(h: np.ndarray) -> np.ndarray:
    return np.asarray(h, dtype=np.uint16).view(np.float16).astype(np.float32)


def frame(scene, nthreads=1, precision=32, rows=None, row_step=1, shadowmap=None, gbuf=None, warp_mode=0,
          warp_high=2.0, warp_low=0.5, tesselation=False, max_tess_level=64.0, **trace_over):
    """The whole reference pipeline on the CPU (voxelize, normalise, inject,
    mips, trace), optionally warped (warp_mode 1: about the eye; 2: through
    the warp map of the scene's 32^3 occupancy; 3: the perspective warp),
    with the rasterising or (tesselation=True) the tessellation voxeliser.
    Returns a dict of every intermediate."""
    sm = render_shadowmap(scene, nthreads) if shadowmap is None else shadowmap
    wmap = None
    if warp_mode == 2:
        wmap = warpmap(warp_occupancy(scene, sm, nthreads), warp_high, warp_low)
    w = warp(scene, warp_mode, wmap) if warp_mode else None
    if tesselation:
        count, sums, total = voxelize_tess(scene, max_tess_level, nthreads=nthreads, warp=w)
    else:
        count, sums, total = voxelize(scene, sm, nthreads=nthreads, warp=w)
    nv = scene.dim ** 3
    chain = np.zeros(4 * chain_voxels(scene.dim, scene.levels), dtype=np.uint16)
    color, normal, _, stats = normalize(scene, count, sums, radiance=chain, nthreads=nthreads)
    inject(scene, sm, color, normal, chain, nthreads=nthreads, warp=w)
    build_mips(scene.dim, scene.levels, chain, nthreads)
    gp, gn, ga = render_gbuffer(scene) if gbuf is None else gbuf
    irr, spec, col, ns = trace(scene, chain, gp, gn, ga, precision=precision, rows=rows, row_step=row_step,
                               nthreads=nthreads, warp=w, **trace_over)
    stats["total_voxel_fragments"] = total
    return dict(shadowmap=sm, count=count, sums=sums, color=color, normal=normal, chain=chain, gpos=gp, gnrm=gn,
                galb=ga, irradiance=irr, specular=spec, out=col, samples=ns, stats=stats, nv=nv, warpmap=wmap,
                warp=w)


# ------------------------------------------------------------ learned path
def cone_set16() -> np.ndarray:
    """The learned path's 16-cone reference set, (16, 4) float32: Fibonacci
    hemisphere directions z_i = 1 - (i + 1/2)/16, azimuth i * golden angle,
    in the (T, B, N) frame, weights cos(theta) / sum cos(theta)."""
    golden = np.pi * (3.0 - np.sqrt(5.0))
    i = np.arange(16, dtype=np.float64)
    z = 1.0 - (i + 0.5) / 16.0
    r = np.sqrt(1.0 - z * z)
    d = np.stack([r * np.cos(golden * i), r * np.sin(golden * i), z, z / z.sum()], 1)
    return d.astype(np.float32)


def reference16_cone(scene) -> orc_cone:
    """Cone settings of the 16-cone reference: the diffuse cone's bias,
    initial height and LOD offset, 24 steps, aperture 2 acos(15/16)."""
    steps, ang, bias, h0, lod = scene.cone["diffuse"]
    return orc_cone(24, float(np.float32(2.0 * np.arccos(15.0 / 16.0))), float(bias), float(h0), float(lod))


def trace_reference16(scene, chain, gpos, gnrm, pixels, precision=64, nthreads=1):
    """16-cone irradiance (float4) at the listed pixels (y * width + x)."""
    W, H = scene.gbuffer_size
    pixels = np.ascontiguousarray(pixels, dtype=np.int32)
    out = np.zeros((pixels.size, 4), dtype=np.float32)
    dirs = cone_set16()
    cone = reference16_cone(scene)
    samples = C.c_uint64(0)
    load().orc_trace_cone_set(C.byref(volume(scene)), scene.levels, _p(chain), _p(dirs), 16, C.byref(cone),
                              C.c_float(float(np.sqrt(3.0))), _p(gpos), _p(gnrm), W, _p(pixels),
                              C.c_int64(pixels.size), precision, _p(out), C.byref(samples), nthreads, None)
    return out, int(samples.value)


def learned_features(scene, chain, gpos, gnrm) -> np.ndarray:
    """Cheap quarter-resolution features (fp32), (ceil(H/4) * ceil(W/4), 32)."""
    W, H = scene.gbuffer_size
    wq, hq = (W + 3) // 4, (H + 3) // 4
    out = np.zeros((hq * wq, 32), dtype=np.float32)
    load().orc_learned_features(C.byref(volume(scene)), scene.levels, _p(chain), _p(gpos), _p(gnrm), W, H, _p(out),
                                None)
    return out


# ----------------------------------------------------- dynamic scenes
def decay_radiance(radiance: np.ndarray, decay: float) -> np.ndarray:
    """temporalRadianceFilter.comp on a level-0 radiance array (in place)."""
    load().orc_decay_radiance(_p(radiance), C.c_int64(radiance.size // 4), C.c_float(decay))
    return radiance


def normal_matrix(model: np.ndarray) -> np.ndarray:
    out = np.zeros(9, dtype=np.float32)
    load().orc_normal_matrix(_f(np.asarray(model, np.float32).reshape(16), 16), _p(out))
    return out


def transform_actors(positions, normals, first, count, models):
    """World-space copies of positions / normals (T x 9 float32) with the
    listed triangle ranges transformed by their column-major models."""
    pos = np.ascontiguousarray(positions, dtype=np.float32).copy()
    nrm = np.ascontiguousarray(normals, dtype=np.float32).copy()
    f = np.ascontiguousarray(first, dtype=np.int64)
    c = np.ascontiguousarray(count, dtype=np.int64)
    m = np.ascontiguousarray(models, dtype=np.float32).reshape(-1, 16)
    load().orc_transform_actors(_p(np.ascontiguousarray(positions, dtype=np.float32)),
                                _p(np.ascontiguousarray(normals, dtype=np.float32)), _p(f), _p(c), _p(m), len(f),
                                _p(pos), _p(nrm))
    return pos, nrm


def shade(scene, gbuf, shadowmap, irradiance=None, specular=None, eye=None, **params):
    """phong.frag's composite with direct lighting; params: the
    orc_shade_params fields (defaults: Cook-Torrance, roughness 0.5,
    metallic 0, shininess 32, the trace's composite switches on, ambient and
    reflect scale 1)."""
    W, H = scene.gbuffer_size
    d = dict(cooktorrance=1, enable_diffuse=1, enable_specular=1, enable_indirect=1, enable_reflections=1,
             draw_occlusion=1, enable_postprocess=1, roughness=0.5, metallic=0.0, shininess=32.0, ambient_scale=1.0,
             reflect_scale=1.0)
    d.update(params)
    sp = orc_shade_params(**d)
    gp, gn, ga = (np.ascontiguousarray(a, dtype=np.float32) for a in gbuf)
    arr, n = lights(scene)
    sw, sh = scene.shadow_size
    out = np.zeros(W * H * 4, dtype=np.float32)
    ir = None if irradiance is None else np.ascontiguousarray(irradiance, dtype=np.float32)
    spc = None if specular is None else np.ascontiguousarray(specular, dtype=np.float32)
    load().orc_shade(_p(gp), _p(gn), _p(ga), W, H, _f(scene.eye if eye is None else eye, 3), arr, n,
                     _p(np.ascontiguousarray(shadowmap, dtype=np.float32)), sw, sh, _f(scene.ls, 16), _p(ir), _p(spc),
                     C.byref(sp), _p(out))
    return out
