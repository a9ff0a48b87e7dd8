"""ctypes binding of the C ABI in include/vct.h (libvct.so, built in-tree).

Loading fails loudly when the library has not been built: there is no CPU
or pure-Python fallback for the hot path.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvct.so")

VCT_OK = 0
VCT_ERR_INVALID_ARGUMENT = 1
VCT_ERR_OUT_OF_MEMORY = 2
VCT_ERR_CUDA = 3
VCT_ERR_STATE = 4
VCT_ERR_TIMEOUT = 5
VCT_ERR_UNSUPPORTED = 6
VCT_ERR_OVERFLOW = 7

VCT_LIGHT_POINT = 0
VCT_LIGHT_DIRECTIONAL = 1
VCT_CONFIG_COLOR_MIPS = 1
VCT_FILTER_SOFTWARE = 0
VCT_FILTER_HARDWARE = 1
VCT_FILTER_HARDWARE_LEVELS = 2
VCT_FILTER_HYBRID = 3
VCT_WARP_NONE = 0
VCT_WARP_ANALYTIC = 1
VCT_WARP_TEXTURE = 2
VCT_WARP_PERSPECTIVE = 3
VCT_WARP_DIM = 32
VCT_MAX_TESS_LEVEL = 64
VCT_MAX_ACTORS = 64
VCT_VOLUME_COLOR = 0
VCT_VOLUME_NORMAL = 1
VCT_VOLUME_RADIANCE = 2
VCT_MAX_LIGHTS = 16
VCT_STATS_COUNT_OVERFLOW = 1

f3 = C.c_float * 3
f16 = C.c_float * 16


class vct_light(C.Structure):
    _fields_ = [
        ("position", f3), ("_pad0", C.c_float),
        ("direction", f3), ("_pad1", C.c_float),
        ("color", f3), ("range", C.c_float), ("intensity", C.c_float),
        ("enabled", C.c_uint32), ("selected", C.c_uint32), ("shadow_caster", C.c_uint32),
        ("type", C.c_uint32), ("_pad2", C.c_uint32 * 3),
    ]


class vct_config(C.Structure):
    _fields_ = [
        ("voxel_dim", C.c_int32), ("voxel_levels", C.c_int32),
        ("voxel_min", f3), ("voxel_max", f3), ("voxel_center", f3),
        ("device", C.c_int32), ("flags", C.c_uint32),
    ]


class vct_cone_settings(C.Structure):
    _fields_ = [("steps", C.c_int32), ("cone_angle", C.c_float), ("bias", C.c_float),
                ("cone_initial_height", C.c_float), ("lod_offset", C.c_float)]


class vct_params(C.Structure):
    _fields_ = [
        ("voxelize_lighting", C.c_int32), ("axis_override", C.c_int32),
        ("voxel_set_opacity", C.c_float), ("temporal_filter", C.c_int32), ("temporal_decay", C.c_float),
        ("radiance_lighting", C.c_int32), ("radiance_dilate", C.c_int32),
        ("diffuse_cone", vct_cone_settings), ("specular_cone", vct_cone_settings),
        ("enable_indirect", C.c_int32), ("enable_reflections", C.c_int32),
        ("draw_occlusion", C.c_int32), ("enable_postprocess", C.c_int32),
        ("ambient_scale", C.c_float), ("reflect_scale", C.c_float), ("max_distance", C.c_float),
        ("ref_tbn_quirk", C.c_int32), ("trace_filter", C.c_int32),
        ("warp_mode", C.c_int32), ("warp_high_resolution", C.c_float), ("warp_low_resolution", C.c_float),
        ("cooktorrance", C.c_int32), ("enable_diffuse", C.c_int32), ("enable_specular", C.c_int32),
        ("roughness", C.c_float), ("metallic", C.c_float), ("shininess", C.c_float),
        ("voxelize_tesselation", C.c_int32), ("max_tess_level", C.c_float), ("pv", f16),
    ]


class vct_triangles(C.Structure):
    _fields_ = [("positions_dev", C.c_void_p), ("normals_dev", C.c_void_p), ("albedo_dev", C.c_void_p),
                ("count", C.c_int64)]


class vct_gbuffer(C.Structure):
    _fields_ = [("position_dev", C.c_void_p), ("normal_dev", C.c_void_p), ("albedo_dev", C.c_void_p),
                ("width", C.c_int32), ("height", C.c_int32)]


class vct_trace_out(C.Structure):
    _fields_ = [("irradiance_dev", C.c_void_p), ("specular_dev", C.c_void_p), ("color_dev", C.c_void_p),
                ("sample_count_dev", C.c_void_p)]


class vct_shadow_desc(C.Structure):
    _fields_ = [("shadowmap_dev", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32),
                ("ls", f16), ("ls_inverse", f16), ("light_pos", f3), ("light_int", f3)]


class vct_timers(C.Structure):
    _fields_ = [("voxelize_ms", C.c_float), ("radiance_ms", C.c_float), ("mipmap_ms", C.c_float),
                ("render_ms", C.c_float), ("total_ms", C.c_float)]


class vct_stats(C.Structure):
    _fields_ = [("total_voxel_fragments", C.c_uint32), ("unique_voxels", C.c_uint32),
                ("max_fragments_per_voxel", C.c_uint32), ("error_flags", C.c_uint32)]


class vct_tuning(C.Structure):
    _fields_ = [("voxel_unit_pixels", C.c_int32), ("voxel_blocks_per_sm", C.c_int32), ("trace_tile_w", C.c_int32),
                ("trace_tile_h", C.c_int32), ("trace_warp_w", C.c_int32)]


class vct_actor(C.Structure):
    _fields_ = [("first_triangle", C.c_int64), ("triangle_count", C.c_int64), ("model", C.c_float * 16)]


class vct_adam(C.Structure):
    _fields_ = [("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float)]


class vct_learned_stats(C.Structure):
    _fields_ = [("tiles", C.c_int32), ("fallback_tiles", C.c_int32), ("mean_tile_error", C.c_float),
                ("max_tile_error", C.c_float)]


class vct_scene_desc(C.Structure):
    _fields_ = [("triangles", vct_triangles), ("lights", C.POINTER(vct_light)), ("n_lights", C.c_int32),
                ("shadow", vct_shadow_desc), ("eye", C.c_float * 3), ("gbuffer", vct_gbuffer),
                ("out", vct_trace_out)]


P = C.POINTER
vp = C.c_void_p
st = C.c_int

# name -> (restype, argtypes); every symbol declared in include/vct.h.
SIGNATURES = {
    "vct_abi_version": (C.c_int32, []),
    "vct_status_string": (C.c_char_p, [st]),
    "vct_last_error": (C.c_char_p, []),
    "vct_struct_sizes": (None, [P(C.c_int64)] * 8),
    "vct_struct_layout": (C.c_int64, [C.c_char_p]),
    "vct_default_params": (None, [P(vct_params)]),
    "vct_voxel_mvp": (st, [P(vct_config), P(C.c_float)]),
    "vct_create": (st, [P(vct_config), P(vp)]),
    "vct_destroy": (st, [vp]),
    "vct_set_params": (st, [vp, P(vct_params)]),
    "vct_get_params": (st, [vp, P(vct_params)]),
    "vct_get_config": (st, [vp, P(vct_config)]),
    "vct_volume_level": (st, [vp, C.c_int32, C.c_int32, P(vp), P(C.c_int32)]),
    "vct_accumulators": (st, [vp, P(vp), P(vp)]),
    "vct_record_slot": (C.c_int64, [C.c_int64, C.c_int32]),
    "vct_voxelize_accumulate": (st, [vp, P(vct_triangles), P(vct_light), C.c_int32, P(vct_shadow_desc),
                                     P(C.c_float), vp]),
    "vct_normalize": (st, [vp, vp]),
    "vct_clear_accumulators": (st, [vp, vp]),
    "vct_voxelize": (st, [vp, P(vct_triangles), P(vct_light), C.c_int32, P(vct_shadow_desc), P(C.c_float), vp]),
    "vct_inject": (st, [vp, P(vct_shadow_desc), P(C.c_float), vp]),
    "vct_build_mips": (st, [vp, C.c_int32, vp]),
    "vct_trace": (st, [vp, P(vct_gbuffer), P(C.c_float), P(vct_trace_out), vp]),
    "vct_trace_views": (st, [vp, C.c_int32, P(vct_gbuffer), P(C.c_float), P(vct_trace_out), vp]),
    "vct_frame": (st, [vp, P(vct_triangles), P(vct_light), C.c_int32, P(vct_shadow_desc), P(C.c_float),
                       P(vct_gbuffer), P(vct_trace_out), vp]),
    "vct_frame_volume": (st, [vp, P(vct_triangles), P(vct_light), C.c_int32, P(vct_shadow_desc), P(C.c_float), vp]),
    "vct_sampler_rate": (st, [vp, C.c_int32, C.c_int64, P(C.c_double), vp]),
    "vct_get_stats": (st, [vp, P(vct_stats), vp]),
    "vct_enable_timers": (st, [vp, C.c_int32]),
    "vct_get_timers": (st, [vp, P(vct_timers)]),
    "vct_launch_count": (C.c_uint64, []),
    "vct_warpmap": (st, [vp, P(vp)]),
    "vct_decay_radiance": (st, [vp, vp]),
    "vct_shade": (st, [vp, P(vct_gbuffer), P(C.c_float), P(vct_light), C.c_int32, P(vct_shadow_desc), vp, vp, vp,
                       vp]),
    "vct_transform_actors": (st, [P(vct_triangles), P(vct_actor), C.c_int32, vp, vp, vp]),
    "vct_voxelize_static": (st, [P(vct_config), P(vct_params), P(vct_triangles), P(vct_light), C.c_int32,
                                 P(vct_shadow_desc), vp, vp, vp, P(vct_stats), vp]),
    "vct_render_shadowmap": (st, [P(vct_triangles), P(C.c_float), vp, C.c_int32, C.c_int32, vp]),
    "vct_render_gbuffer": (st, [P(vct_triangles), P(C.c_float), P(C.c_float), P(C.c_float), C.c_int32, C.c_int32,
                                vp, vp, vp, vp, vp]),
    "vct_batch_create": (st, [P(vct_config), C.c_int32, P(vp)]),
    "vct_batch_destroy": (st, [vp]),
    "vct_batch_set_params": (st, [vp, C.c_int32, P(vct_params)]),
    "vct_batch_frame": (st, [vp, P(vct_scene_desc), C.c_int32, vp]),
    "vct_batch_capture": (st, [vp, P(vct_scene_desc), C.c_int32, vp]),
    "vct_batch_replay": (st, [vp, vp]),
    "vct_batch_context": (st, [vp, C.c_int32, P(vp)]),
    "vct_batch_enable_timers": (st, [vp, C.c_int32]),
    "vct_batch_get_timers": (st, [vp, P(vct_timers)]),
    "vct_tensor_core_check": (st, [vp, vp, C.c_int32, C.c_int32, C.c_int32, vp, vp]),
    "vct_timeout_probe": (st, [C.c_int64, vp]),
    "vct_mlp_create": (st, [C.c_int32, C.c_uint64, P(vp)]),
    "vct_mlp_destroy": (st, [vp]),
    "vct_mlp_set_params": (st, [vp, P(C.c_float), C.c_int64]),
    "vct_mlp_get_params": (st, [vp, P(C.c_float), C.c_int64, vp]),
    "vct_mlp_forward": (st, [vp, vp, C.c_int64, vp, vp]),
    "vct_mlp_gradients": (st, [vp, vp, vp, C.c_int64, vp, vp, vp]),
    "vct_mlp_train_step": (st, [vp, vp, vp, vp, C.c_int64, P(vct_adam), vp, vp]),
    "vct_learned_features": (st, [vp, P(vct_gbuffer), P(C.c_float), vp, vp]),
    "vct_learned_rows": (st, [vp, P(vct_gbuffer), P(C.c_float), vp, vp, C.c_int64, vp, vp]),
    "vct_trace_reference16": (st, [vp, P(vct_gbuffer), P(C.c_float), vp, vp]),
    "vct_learned_trace": (st, [vp, vp, P(vct_gbuffer), P(C.c_float), C.c_float, vp, P(vct_learned_stats), vp]),
    "vct_learned_trace_pixels": (st, [vp, vp, P(vct_gbuffer), P(C.c_float), C.c_float, vp, P(C.c_int64), vp]),
    "vct_default_tuning": (None, [P(vct_tuning)]),
    "vct_get_tuning": (st, [vp, P(vct_tuning)]),
    "vct_set_tuning": (st, [vp, P(vct_tuning)]),
    "vct_batch_get_tuning": (st, [vp, P(vct_tuning)]),
    "vct_batch_set_tuning": (st, [vp, P(vct_tuning)]),
    "vct_autotune": (st, [vp, P(vct_triangles), P(vct_light), C.c_int32, P(vct_shadow_desc), P(C.c_float),
                          P(vct_gbuffer), P(vct_trace_out), C.c_int32, vp, P(vct_tuning)]),
    "vct_batch_autotune": (st, [vp, P(vct_scene_desc), C.c_int32, C.c_int32, vp, P(vct_tuning)]),
}

_lib = None


class VctError(RuntimeError):
    def __init__(self, status: int, func: str, msg: str):
        super().__init__(f"{func} failed with status {status}: {msg}")
        self.status = status


def load() -> C.CDLL:
    """Load libvct.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                           " (there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, func: str) -> None:
    if status != VCT_OK:
        lib = load()
        raise VctError(status, func, (lib.vct_last_error() or b"").decode())


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
