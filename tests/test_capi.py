"""C ABI checks that need no GPU: the library loads, exports every entry
point include/vct.h declares, its struct layouts match the FFI binding, its
defaults are the reference's, and argument validation fails loudly before
any device work."""

from __future__ import annotations

import ctypes as C
import math
import os
import re

import numpy as np

import oracle as O
from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "vct.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(vct_\w+)\s*\(", src, flags=re.M)))


def test_every_declared_symbol_is_exported_and_bound():
    lib = C.CDLL(L.LIB_PATH)
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
        assert n in L.SIGNATURES, f"{n} missing from the ctypes binding"
    assert set(L.SIGNATURES) == set(names)


def test_struct_layouts_match():
    lib = L.load()
    sz = [C.c_int64() for _ in range(8)]
    lib.vct_struct_sizes(*[C.byref(s) for s in sz])
    py = [L.vct_light, L.vct_config, L.vct_params, L.vct_triangles, L.vct_gbuffer, L.vct_trace_out,
          L.vct_shadow_desc, L.vct_stats]
    assert [s.value for s in sz] == [C.sizeof(t) for t in py]
    # std140 light record of the reference (src/Scene.cpp:64-76)
    assert C.sizeof(L.vct_light) == 80
    assert L.vct_light.range.offset == 44 and L.vct_light.intensity.offset == 48
    assert L.vct_light.enabled.offset == 52 and L.vct_light.shadow_caster.offset == 60
    assert L.vct_light.type.offset == 64
    assert lib.vct_abi_version() == 1


def test_default_params_are_reference_defaults():
    p = api.default_params()
    # src/Application.h:36-103
    assert p.voxelize_lighting == 1 and p.axis_override == -1
    assert p.voxel_set_opacity == np.float32(0.5) and p.temporal_filter == 0
    assert p.temporal_decay == np.float32(0.8)
    assert p.radiance_lighting == 0 and p.radiance_dilate == 0
    d, s = p.diffuse_cone, p.specular_cone
    assert (d.steps, s.steps) == (16, 32)
    assert math.isclose(d.cone_angle, math.radians(60), rel_tol=1e-6)
    assert math.isclose(s.cone_angle, math.radians(30), rel_tol=1e-6)
    assert (d.bias, d.cone_initial_height, d.lod_offset) == (1.0, 1.0, 0.5)
    assert np.allclose((s.bias, s.cone_initial_height, s.lod_offset), (1.7, 0.5, 0.1))
    assert p.enable_indirect == p.enable_reflections == p.draw_occlusion == p.enable_postprocess == 1
    assert p.ambient_scale == 1.0 and p.reflect_scale == 1.0
    assert p.trace_filter == L.VCT_FILTER_SOFTWARE


def test_voxel_mvp_equals_oracle_bitwise():
    lib = L.load()
    for vmax, center in ((1.0, (0, 0, 0)), (20.0, (0, 0, 0)), (3.5, (1.25, -2.0, 0.5))):
        sc = scenes.tiny()
        sc.vmax = vmax
        cfg = api.config_for(sc)
        cfg.voxel_center = api.f3(center)
        out = (C.c_float * 48)()
        L.check(lib.vct_voxel_mvp(C.byref(cfg), out), "vct_voxel_mvp")
        vol = O.volume(sc)
        vol.vcenter = (C.c_float * 3)(*center)
        ref = np.zeros(48, np.float32)
        O.load().orc_voxel_mvp(C.byref(vol), ref.ctypes.data_as(C.c_void_p))
        assert np.array_equal(np.frombuffer(out, np.float32), ref)


def test_invalid_configs_rejected_before_device_work():
    lib = L.load()
    sc = scenes.tiny()
    h = C.c_void_p()
    for mutate, msg in ((lambda c: setattr(c, "voxel_dim", 48), b"power of two"),
                        (lambda c: setattr(c, "voxel_dim", 8), b"power of two"),
                        (lambda c: setattr(c, "voxel_dim", 2048), b"power of two"),
                        (lambda c: setattr(c, "voxel_min", api.f3([-1, -2, -1])), b"symmetric"),
                        (lambda c: setattr(c, "voxel_max", api.f3([1, 2, 1])), b""),
                        (lambda c: setattr(c, "voxel_levels", -1), b"voxel_levels")):
        cfg = api.config_for(sc)
        mutate(cfg)
        rc = lib.vct_create(C.byref(cfg), C.byref(h))
        assert rc == L.VCT_ERR_INVALID_ARGUMENT
        assert msg in lib.vct_last_error()
    assert lib.vct_create(None, C.byref(h)) == L.VCT_ERR_INVALID_ARGUMENT
    assert lib.vct_set_params(None, None) == L.VCT_ERR_INVALID_ARGUMENT
    assert lib.vct_destroy(None) == L.VCT_OK


def test_status_strings():
    lib = L.load()
    for code in range(8):
        assert lib.vct_status_string(code)
    assert lib.vct_status_string(L.VCT_OK) == b"ok"


def test_static_entry_point_rejects_before_device_work():
    lib = L.load()
    sc = scenes.tiny()
    params = api.scene_params(sc)
    cfg = api.config_for(sc, dim=128)
    tris = L.vct_triangles()
    lights, n = api.light_array(sc.lights)
    rc = lib.vct_voxelize_static(C.byref(cfg), C.byref(params), C.byref(tris), lights, n, None, None, None, None,
                                 None, None)
    # the shadow caster needs a shadow description: rejected first
    assert rc == L.VCT_ERR_INVALID_ARGUMENT


def test_default_tuning_and_scene_desc_layout():
    t = L.vct_tuning()
    L.load().vct_default_tuning(C.byref(t))
    assert api.tuning_dict(t) == dict(voxel_unit_pixels=512, voxel_blocks_per_sm=3, trace_tile_w=16, trace_tile_h=16,
                                      trace_warp_w=8)
    lib = L.load()
    for cls in (L.vct_light, L.vct_config, L.vct_cone_settings, L.vct_params, L.vct_triangles, L.vct_gbuffer,
                L.vct_trace_out, L.vct_shadow_desc, L.vct_stats, L.vct_timers, L.vct_tuning, L.vct_scene_desc,
                L.vct_adam, L.vct_learned_stats):
        assert lib.vct_struct_layout(cls.__name__.encode()) == C.sizeof(cls), cls.__name__
    for f in ("lights", "n_lights", "shadow", "eye", "gbuffer", "out"):
        assert lib.vct_struct_layout(f"vct_scene_desc.{f}".encode()) == getattr(L.vct_scene_desc, f).offset, f
    assert lib.vct_struct_layout(b"vct_params.trace_filter") == L.vct_params.trace_filter.offset
    assert lib.vct_struct_layout(b"vct_tuning.trace_warp_w") == L.vct_tuning.trace_warp_w.offset
    assert lib.vct_struct_layout(b"vct_learned_stats.max_tile_error") == L.vct_learned_stats.max_tile_error.offset
    assert lib.vct_struct_layout(b"no_such_struct") == -1
