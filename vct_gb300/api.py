"""Python mirror of the C ABI, for tests and benchmarks.

Device buffers are torch CUDA tensors (torch is only the allocator and stream
provider here); every call goes straight to the C entry point of the same
name in libvct.so.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _ptr(t) -> int:
    if t is None:
        return 0
    if isinstance(t, int):
        return t
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return int(t.data_ptr())


def _stream(stream) -> int:
    if stream is None:
        import torch

        return int(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)


def f3(v) -> C.Array:
    a = np.asarray(v, dtype=np.float32).reshape(3)
    return (C.c_float * 3)(*a.tolist())


def f16(v) -> C.Array:
    a = np.asarray(v, dtype=np.float32).reshape(16)
    return (C.c_float * 16)(*a.tolist())


def default_params() -> L.vct_params:
    p = L.vct_params()
    L.load().vct_default_params(C.byref(p))
    return p


def scene_params(scene, **overrides) -> L.vct_params:
    """Reference defaults with the scene's cone settings and overrides."""
    p = default_params()
    for key, name in (("diffuse", "diffuse_cone"), ("specular", "specular_cone")):
        if key in scene.cone:
            steps, ang, bias, h0, lod = scene.cone[key]
            setattr(p, name, L.vct_cone_settings(int(steps), float(ang), float(bias), float(h0), float(lod)))
    p.max_distance = float(np.sqrt(3.0))  # grid diagonal in texture units
    if getattr(scene, "pv", None) is not None:
        p.pv = (C.c_float * 16)(*np.asarray(scene.pv, dtype=np.float32).tolist())
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def light_array(lights) -> tuple:
    arr = (L.vct_light * max(1, len(lights)))()
    for i, d in enumerate(lights):
        li = arr[i]
        li.position = f3(d["position"])
        li.direction = f3(d["direction"])
        li.color = f3(d["color"])
        li.range = float(d["range"])
        li.intensity = float(d["intensity"])
        li.enabled = int(d.get("enabled", 1))
        li.shadow_caster = int(d.get("shadow_caster", 0))
        li.type = int(d["type"])
    return arr, len(lights)


def config_for(scene, device: int = 0, flags: int = 0, dim: int | None = None) -> L.vct_config:
    c = L.vct_config()
    c.voxel_dim = int(dim or scene.dim)
    c.voxel_levels = 0
    c.voxel_min = f3([-scene.vmax] * 3)
    c.voxel_max = f3([scene.vmax] * 3)
    c.voxel_center = f3([0, 0, 0])
    c.device = device
    c.flags = flags
    return c


def triangles(pos, nrm, alb) -> L.vct_triangles:
    t = L.vct_triangles()
    t.positions_dev = _ptr(pos)
    t.normals_dev = _ptr(nrm)
    t.albedo_dev = _ptr(alb)
    t.count = int(pos.shape[0]) if pos is not None else 0
    return t


def shadow_desc(scene, shadowmap) -> L.vct_shadow_desc:
    s = L.vct_shadow_desc()
    s.shadowmap_dev = _ptr(shadowmap)
    s.width, s.height = scene.shadow_size
    s.ls = f16(scene.ls)
    s.ls_inverse = f16(scene.ls_inverse)
    s.light_pos = f3(scene.light_pos)
    s.light_int = f3(scene.light_int)
    return s


def gbuffer(gpos, gnrm, galb, width: int, height: int) -> L.vct_gbuffer:
    g = L.vct_gbuffer()
    g.position_dev, g.normal_dev, g.albedo_dev = _ptr(gpos), _ptr(gnrm), _ptr(galb)
    g.width, g.height = width, height
    return g


def trace_out(irradiance=None, specular=None, color=None, samples=None) -> L.vct_trace_out:
    o = L.vct_trace_out()
    o.irradiance_dev, o.specular_dev, o.color_dev = _ptr(irradiance), _ptr(specular), _ptr(color)
    o.sample_count_dev = _ptr(samples)
    return o


class Context:
    """Owns a vct_ctx (volumes on one device); with `handle`, a view of a
    context owned by a Batch, never destroyed through the view."""

    def __init__(self, config: L.vct_config | None = None, *, handle: C.c_void_p | None = None):
        self._lib = L.load()
        self._owned = handle is None
        if handle is None:
            h = C.c_void_p()
            L.check(self._lib.vct_create(C.byref(config), C.byref(h)), "vct_create")
        else:
            h = handle
        self.handle = h
        cfg = L.vct_config()
        L.check(self._lib.vct_get_config(h, C.byref(cfg)), "vct_get_config")
        self.dim = cfg.voxel_dim
        self.levels = cfg.voxel_levels

    def close(self):
        if getattr(self, "handle", None):
            if self._owned:
                self._lib.vct_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_params(self, p: L.vct_params):
        L.check(self._lib.vct_set_params(self.handle, C.byref(p)), "vct_set_params")

    def get_params(self) -> L.vct_params:
        p = L.vct_params()
        L.check(self._lib.vct_get_params(self.handle, C.byref(p)), "vct_get_params")
        return p

    def voxelize_accumulate(self, tris, lights, shadow, eye, stream=None):
        arr, n = lights
        L.check(self._lib.vct_voxelize_accumulate(self.handle, C.byref(tris), arr, n, C.byref(shadow), f3(eye),
                                                   _stream(stream)), "vct_voxelize_accumulate")

    def normalize(self, stream=None):
        L.check(self._lib.vct_normalize(self.handle, _stream(stream)), "vct_normalize")

    def voxelize(self, tris, lights, shadow, eye, stream=None):
        arr, n = lights
        L.check(self._lib.vct_voxelize(self.handle, C.byref(tris), arr, n, C.byref(shadow), f3(eye), _stream(stream)),
                "vct_voxelize")

    def inject(self, shadow, eye, stream=None):
        L.check(self._lib.vct_inject(self.handle, C.byref(shadow), f3(eye), _stream(stream)), "vct_inject")

    def build_mips(self, volume: int = L.VCT_VOLUME_RADIANCE, stream=None):
        L.check(self._lib.vct_build_mips(self.handle, volume, _stream(stream)), "vct_build_mips")

    def trace(self, gb, eye, out, stream=None):
        L.check(self._lib.vct_trace(self.handle, C.byref(gb), f3(eye), C.byref(out), _stream(stream)), "vct_trace")

    def trace_views(self, gbs, eyes, outs, stream=None):
        """vct_trace_views: the trace of several viewpoints in one launch."""
        n = len(gbs)
        g = (L.vct_gbuffer * max(1, n))(*gbs)
        e = (C.c_float * max(3, 3 * n))(*[float(v) for eye in eyes for v in eye])
        o = (L.vct_trace_out * max(1, n))(*outs)
        L.check(self._lib.vct_trace_views(self.handle, n, g, e, o, _stream(stream)), "vct_trace_views")

    def frame(self, tris, lights, shadow, eye, gb, out, stream=None):
        arr, n = lights
        L.check(self._lib.vct_frame(self.handle, C.byref(tris), arr, n, C.byref(shadow), f3(eye), C.byref(gb),
                                    C.byref(out), _stream(stream)), "vct_frame")

    def frame_volume(self, tris, lights, shadow, eye, stream=None):
        arr, n = lights
        L.check(self._lib.vct_frame_volume(self.handle, C.byref(tris), arr, n, C.byref(shadow), f3(eye),
                                           _stream(stream)), "vct_frame_volume")

    def sampler_rate(self, filt: int, samples: int = 1 << 31, stream=None) -> float:
        r = C.c_double()
        L.check(self._lib.vct_sampler_rate(self.handle, int(filt), int(samples), C.byref(r), _stream(stream)),
                "vct_sampler_rate")
        return r.value

    def enable_timers(self, on: bool = True):
        L.check(self._lib.vct_enable_timers(self.handle, int(on)), "vct_enable_timers")

    def tuning(self) -> L.vct_tuning:
        t = L.vct_tuning()
        L.check(self._lib.vct_get_tuning(self.handle, C.byref(t)), "vct_get_tuning")
        return t

    def set_tuning(self, t: L.vct_tuning):
        L.check(self._lib.vct_set_tuning(self.handle, C.byref(t)), "vct_set_tuning")

    def autotune(self, tris, lights, shadow, eye, gb, out, reps: int = 3, stream=None) -> L.vct_tuning:
        arr, n = lights
        t = L.vct_tuning()
        L.check(self._lib.vct_autotune(self.handle, C.byref(tris), arr, n, C.byref(shadow), f3(eye), C.byref(gb),
                                       C.byref(out), reps, _stream(stream), C.byref(t)), "vct_autotune")
        return t

    def timers(self) -> dict:
        t = L.vct_timers()
        L.check(self._lib.vct_get_timers(self.handle, C.byref(t)), "vct_get_timers")
        return {k: getattr(t, k) for k, _ in L.vct_timers._fields_}

    def stats(self, stream=None) -> dict:
        s = L.vct_stats()
        L.check(self._lib.vct_get_stats(self.handle, C.byref(s), _stream(stream)), "vct_get_stats")
        return dict(total_voxel_fragments=s.total_voxel_fragments, unique_voxels=s.unique_voxels,
                    max_fragments_per_voxel=s.max_fragments_per_voxel, error_flags=s.error_flags)

    def volume_ptr(self, volume: int, level: int) -> tuple[int, int]:
        p = C.c_void_p()
        d = C.c_int32()
        L.check(self._lib.vct_volume_level(self.handle, volume, level, C.byref(p), C.byref(d)), "vct_volume_level")
        return int(p.value), int(d.value)

    def accumulator_ptrs(self) -> tuple[int, int]:
        a, b = C.c_void_p(), C.c_void_p()
        L.check(self._lib.vct_accumulators(self.handle, C.byref(a), C.byref(b)), "vct_accumulators")
        return int(a.value), int(b.value)

    def shade(self, gb, eye, lights, shadow, color, irradiance=None, specular=None, stream=None):
        arr, n = lights
        L.check(self._lib.vct_shade(self.handle, C.byref(gb), f3(eye), arr, n, C.byref(shadow), _ptr(irradiance),
                                    _ptr(specular), _ptr(color), _stream(stream)), "vct_shade")

    def decay_radiance(self, stream=None):
        L.check(self._lib.vct_decay_radiance(self.handle, _stream(stream)), "vct_decay_radiance")

    def read_warpmap(self):
        """Copy of the warp map of the last VCT_WARP_TEXTURE voxelisation:
        (32^3 * 4,) int16 tensor (RGBA16 unorm bit patterns, x fastest)."""
        p = C.c_void_p()
        L.check(self._lib.vct_warpmap(self.handle, C.byref(p)), "vct_warpmap")
        return device_view(int(p.value), (32 ** 3 * 4,), "<i2").clone()

    # -- copies of device state into torch tensors (test helpers)
    def read_volume(self, volume: int, level: int = 0):
        """Copy of one volume level as an int16 tensor (binary16 bit patterns)."""
        ptr, d = self.volume_ptr(volume, level)
        return device_view(ptr, (d * d * d * 4,), "<i2").clone()

    def read_accumulators(self):
        """Copies of (records [dim^3, 8] in voxel order, occupancy mask) as
        int32 tensors (uint32 bit patterns); record = {count, r, g, b, nx, ny,
        nz, 0}."""
        import torch

        rp, op = self.accumulator_ptrs()
        nv = self.dim ** 3
        rec = device_view(rp, (nv, 8), "<i4")
        slots = torch.from_numpy(record_slots(self.dim)).to(rec.device)
        return rec.index_select(0, slots), device_view(op, ((nv + 31) // 32,), "<i4").clone()


def scene_desc(tris, lights, shadow, eye, gb, out) -> L.vct_scene_desc:
    """vct_scene_desc of one batched scene; `lights` is light_array()'s pair
    (the array must stay alive until the frame or capture call returns)."""
    arr, n = lights
    d = L.vct_scene_desc()
    d.triangles, d.lights, d.n_lights, d.shadow = tris, arr, n, shadow
    d.eye = f3(eye)
    d.gbuffer, d.out = gb, out
    return d


class Batch:
    """Owns a vct_batch: one context per scene, one launch per frame stage."""

    def __init__(self, configs):
        self._lib = L.load()
        n = len(configs)
        arr = (L.vct_config * n)(*configs)
        h = C.c_void_p()
        L.check(self._lib.vct_batch_create(arr, n, C.byref(h)), "vct_batch_create")
        self.handle = h
        self.n = n
        self.scenes = []
        for i in range(n):
            c = C.c_void_p()
            L.check(self._lib.vct_batch_context(h, i, C.byref(c)), "vct_batch_context")
            self.scenes.append(Context(handle=c))

    def close(self):
        if getattr(self, "handle", None):
            self._lib.vct_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p: L.vct_params, scene: int = -1):
        L.check(self._lib.vct_batch_set_params(self.handle, scene, C.byref(p)), "vct_batch_set_params")

    def _descs(self, descs):
        return (L.vct_scene_desc * len(descs))(*descs), len(descs)

    def frame(self, descs, stream=None):
        arr, n = self._descs(descs)
        L.check(self._lib.vct_batch_frame(self.handle, arr, n, _stream(stream)), "vct_batch_frame")

    def capture(self, descs, stream):
        arr, n = self._descs(descs)
        L.check(self._lib.vct_batch_capture(self.handle, arr, n, _stream(stream)), "vct_batch_capture")

    def replay(self, stream=None):
        L.check(self._lib.vct_batch_replay(self.handle, _stream(stream)), "vct_batch_replay")

    def enable_timers(self, on: bool = True):
        L.check(self._lib.vct_batch_enable_timers(self.handle, int(on)), "vct_batch_enable_timers")

    def timers(self) -> dict:
        t = L.vct_timers()
        L.check(self._lib.vct_batch_get_timers(self.handle, C.byref(t)), "vct_batch_get_timers")
        return {k: getattr(t, k) for k, _ in L.vct_timers._fields_}

    def tuning(self) -> L.vct_tuning:
        t = L.vct_tuning()
        L.check(self._lib.vct_batch_get_tuning(self.handle, C.byref(t)), "vct_batch_get_tuning")
        return t

    def set_tuning(self, t: L.vct_tuning):
        L.check(self._lib.vct_batch_set_tuning(self.handle, C.byref(t)), "vct_batch_set_tuning")

    def autotune(self, descs, reps: int = 3, stream=None) -> L.vct_tuning:
        arr, n = self._descs(descs)
        t = L.vct_tuning()
        L.check(self._lib.vct_batch_autotune(self.handle, arr, n, reps, _stream(stream), C.byref(t)),
                "vct_batch_autotune")
        return t


class Mlp:
    """Owns a vct_mlp: the learned path's network (see include/vct.h)."""

    NPARAMS = 11332
    OUTPUTS = 4

    def __init__(self, device: int = 0, seed: int = 0):
        self._lib = L.load()
        h = C.c_void_p()
        L.check(self._lib.vct_mlp_create(device, C.c_uint64(seed), C.byref(h)), "vct_mlp_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self._lib.vct_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, stream=None) -> np.ndarray:
        out = np.zeros(self.NPARAMS, dtype=np.float32)
        L.check(self._lib.vct_mlp_get_params(self.handle, out.ctypes.data_as(C.POINTER(C.c_float)), out.size,
                                             _stream(stream)), "vct_mlp_get_params")
        return out

    def set_params(self, p):
        a = np.ascontiguousarray(p, dtype=np.float32)
        L.check(self._lib.vct_mlp_set_params(self.handle, a.ctypes.data_as(C.POINTER(C.c_float)), a.size),
                "vct_mlp_set_params")

    def forward(self, rows, out, stream=None):
        L.check(self._lib.vct_mlp_forward(self.handle, _ptr(rows), int(rows.shape[0]), _ptr(out), _stream(stream)),
                "vct_mlp_forward")

    def gradients(self, rows, targets, grad, loss=None, stream=None):
        L.check(self._lib.vct_mlp_gradients(self.handle, _ptr(rows), _ptr(targets), int(rows.shape[0]), _ptr(grad),
                                            _ptr(loss), _stream(stream)), "vct_mlp_gradients")

    def train_step(self, rows, targets, index, n: int, lr: float, loss=None, beta1=0.9, beta2=0.999, eps=1e-8,
                   stream=None):
        opt = L.vct_adam(lr, beta1, beta2, eps)
        L.check(self._lib.vct_mlp_train_step(self.handle, _ptr(rows), _ptr(targets), _ptr(index), int(n),
                                             C.byref(opt), _ptr(loss), _stream(stream)), "vct_mlp_train_step")


def learned_features(ctx: Context, gb, eye, features, stream=None):
    L.check(L.load().vct_learned_features(ctx.handle, C.byref(gb), f3(eye), _ptr(features), _stream(stream)),
            "vct_learned_features")


def learned_rows(ctx: Context, gb, eye, features, pixels, rows, stream=None):
    L.check(L.load().vct_learned_rows(ctx.handle, C.byref(gb), f3(eye), _ptr(features), _ptr(pixels),
                                      int(pixels.shape[0]), _ptr(rows), _stream(stream)), "vct_learned_rows")


def trace_reference16(ctx: Context, gb, eye, irradiance, stream=None):
    L.check(L.load().vct_trace_reference16(ctx.handle, C.byref(gb), f3(eye), _ptr(irradiance), _stream(stream)),
            "vct_trace_reference16")


def learned_trace(ctx: Context, mlp: Mlp, gb, eye, irradiance, threshold: float = 0.02, want_stats: bool = False,
                  stream=None):
    st = L.vct_learned_stats() if want_stats else None
    L.check(L.load().vct_learned_trace(ctx.handle, mlp.handle, C.byref(gb), f3(eye), C.c_float(threshold),
                                       _ptr(irradiance), C.byref(st) if st is not None else None, _stream(stream)),
            "vct_learned_trace")
    if st is not None:
        return {k: getattr(st, k) for k, _ in L.vct_learned_stats._fields_}
    return None


def learned_trace_pixels(ctx: Context, mlp: Mlp, gb, eye, irradiance, threshold: float, want_count: bool = False,
                         stream=None):
    """vct_learned_trace_pixels; with want_count, returns the number of
    re-traced pixels (and synchronises the stream)."""
    n = C.c_int64(0)
    L.check(L.load().vct_learned_trace_pixels(ctx.handle, mlp.handle, C.byref(gb), f3(eye), C.c_float(threshold),
                                              _ptr(irradiance), C.byref(n) if want_count else None,
                                              _stream(stream)), "vct_learned_trace_pixels")
    return int(n.value) if want_count else None


def actor_array(actors) -> tuple:
    """actors: iterable of (first_triangle, triangle_count, model) with model a
    4x4 row-major numpy matrix (stored column-major, as glm does)."""
    actors = list(actors)
    arr = (L.vct_actor * max(1, len(actors)))()
    for i, (first, count, model) in enumerate(actors):
        arr[i].first_triangle = int(first)
        arr[i].triangle_count = int(count)
        arr[i].model = f16(np.asarray(model, dtype=np.float64).T.reshape(16))
    return arr, len(actors)


def transform_actors(local_tris, actors, positions, normals, stream=None):
    arr, n = actors if isinstance(actors, tuple) else actor_array(actors)
    L.check(L.load().vct_transform_actors(C.byref(local_tris), arr, n, _ptr(positions), _ptr(normals),
                                          _stream(stream)), "vct_transform_actors")


def tuning_dict(t: L.vct_tuning) -> dict:
    return {k: int(getattr(t, k)) for k, _ in L.vct_tuning._fields_}


def tuning_from(d: dict) -> L.vct_tuning:
    t = L.vct_tuning()
    L.load().vct_default_tuning(C.byref(t))
    for k, v in d.items():
        setattr(t, k, int(v))
    return t


class _CudaArray:
    def __init__(self, ptr: int, shape: tuple, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2, "strides": None}


def record_slots(dim: int) -> np.ndarray:
    """Slot of each voxel's record in vct_accumulators' buffer, in voxel
    order (x fastest): bit 1 of x and bit 0 of y change places, so each
    128-byte line holds a 2 x 2 block of records in x and y."""
    v = np.arange(dim ** 3, dtype=np.int64)
    d = ((v >> 1) ^ ((v & dim) != 0)) & 1
    return v ^ (d * (dim + 2))


def device_view(ptr: int, shape: tuple, typestr: str):
    """Zero-copy torch view of device memory owned by libvct."""
    import torch

    return torch.as_tensor(_CudaArray(ptr, shape, typestr), device="cuda")


def render_shadowmap(tris, scene, out, stream=None):
    W, H = scene.shadow_size
    L.call("vct_render_shadowmap", C.byref(tris), f16(scene.ls), _ptr(out), W, H, _stream(stream))


def render_gbuffer(tris, scene, keys, gpos, gnrm, galb, stream=None):
    W, H = scene.gbuffer_size
    L.call("vct_render_gbuffer", C.byref(tris), f16(scene.view_proj), f3(scene.eye), f16(scene.inv_view_proj), W, H,
           _ptr(keys), _ptr(gpos), _ptr(gnrm), _ptr(galb), _stream(stream))
