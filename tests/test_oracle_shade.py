"""Known answers of the oracle's direct-lighting composite (phong.frag:183-344
and main's composite), derived by hand for one pixel lit head-on: surface
at the origin with normal +y, the eye and the light straight above it, so
that N.L = N.V = N.H = H.V = 1 and every BRDF term has a closed form.

Blinn-Phong (phong.frag:255-263,284-296):
  diffuse = specular = N.L * colour * intensity * albedo   (pow(1, shininess) = 1)
Cook-Torrance (phong.frag:229-253, 528-549), roughness r = 0.5, metallic 0:
  D = r^2 / (PI (r^2 - 1 + 1)^2) = 1 / (PI r^2) = 4 / PI,  G = 1,
  F = 0.04 + 0.96 (1 - 1)^5 = 0.04,  f_ct = D G F / 4 = 0.04 / PI,
  diffuse = colour (1 - F) albedo / PI,  specular = colour 0.04 / PI
  (PI = 3.1415982 as common.glsl:1 spells it; the light's intensity is not
  used by the Cook-Torrance branch).
Composite without the indirect term: ambientScale * albedo + diffuse +
specular; postprocess: c / (c + 1), then ^(1 / 2.2).
Point lights: attenuation 1 - smoothstep(0.75 R, R, d), 0 beyond R.
"""

from __future__ import annotations

import dataclasses

import numpy as np
import pytest

import oracle as O
from vct_gb300 import scenes

PI = np.float64(3.1415982)
ALBEDO = np.array([0.2, 0.4, 0.6])


def _pixel(light, **params):
    sc = dataclasses.replace(scenes.tiny(seed=0), lights=[light], gbuffer_size=(1, 1), shadow_size=(1, 1),
                             eye=np.array([0.0, 2.0, 0.0], np.float32))
    gp = np.array([0.0, 0.0, 0.0, 1.0], np.float32)
    gn = np.array([0.0, 1.0, 0.0, 0.0], np.float32)
    ga = np.array([*ALBEDO, 1.0], np.float32)
    d = dict(enable_indirect=0, enable_postprocess=0)
    d.update(params)
    out = O.shade(sc, (gp, gn, ga), np.ones(1, np.float32), **d)
    return out[:3].astype(np.float64)


def _dir_light(intensity=0.8):
    return dict(position=np.array([0.0, 5.0, 0.0]), direction=np.array([0.0, -1.0, 0.0]), color=np.ones(3),
                range=10.0, intensity=intensity, shadow_caster=0, type=1)


def _point_light(height, rng=2.0, intensity=0.8):
    return dict(position=np.array([0.0, height, 0.0]), direction=np.array([0.0, -1.0, 0.0]), color=np.ones(3),
                range=rng, intensity=intensity, shadow_caster=0, type=0)


def test_blinn_phong_head_on():
    got = _pixel(_dir_light(0.8), cooktorrance=0)
    want = ALBEDO + 0.8 * ALBEDO + 0.8 * ALBEDO
    assert np.allclose(got, want, rtol=1e-6)
    # each term switches off on its own
    assert np.allclose(_pixel(_dir_light(0.8), cooktorrance=0, enable_specular=0), ALBEDO * 1.8, rtol=1e-6)
    assert np.allclose(_pixel(_dir_light(0.8), cooktorrance=0, enable_diffuse=0), ALBEDO * 1.8, rtol=1e-6)


def test_cook_torrance_head_on():
    got = _pixel(_dir_light(0.8), cooktorrance=1, roughness=0.5, metallic=0.0)
    want = ALBEDO + 0.96 * ALBEDO / PI + 0.04 / PI
    assert np.allclose(got, want, rtol=2e-6)


def test_cook_torrance_metallic_head_on():
    # metallic 1: F0 = albedo, F = albedo, kd = 0: only the specular term D G F / 4 = albedo / PI
    got = _pixel(_dir_light(0.8), cooktorrance=1, roughness=0.5, metallic=1.0)
    want = ALBEDO + ALBEDO / PI
    assert np.allclose(got, want, rtol=2e-6)


def test_postprocess_tone_map_and_gamma():
    got = _pixel(_dir_light(0.8), cooktorrance=0, enable_postprocess=1)
    c = ALBEDO * 2.6
    want = (c / (c + 1.0)) ** (1.0 / 2.2)
    assert np.allclose(got, want, rtol=2e-6)


@pytest.mark.parametrize("height,att", [(1.0, 1.0), (1.75, 0.5), (2.5, 0.0)])
def test_point_light_attenuation(height, att):
    # range 2: smoothstep(1.5, 2, d) is 0 at d = 1, 1/2 at d = 1.75; beyond the range the light is skipped
    got = _pixel(_point_light(height), cooktorrance=0)
    want = ALBEDO + att * (0.8 * ALBEDO + 0.8 * ALBEDO)
    assert np.allclose(got, want, rtol=1e-6, atol=1e-7)
