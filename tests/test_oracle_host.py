"""Host-side checks: seeded scenes have the configured shapes, and the
oracle gives bit-identical results for any thread count (the reference arm
of the benchmark runs it on every host core)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from vct_gb300 import scenes


def test_scene_sizes_and_determinism():
    c = scenes.cornell(seed=3)
    assert c.ntri == 10 + 1280 and c.dim == 64 and c.levels == 7
    assert c.shadow_size == (512, 512) and c.gbuffer_size == (640, 360)
    c2 = scenes.cornell(seed=3)
    assert np.array_equal(c.positions, c2.positions) and np.array_equal(c.albedo, c2.albedo)
    assert not np.array_equal(c.positions, scenes.cornell(seed=4).positions)
    n = c.normals.reshape(-1, 3)
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-5)
    assert ((c.albedo >= 0.1) & (c.albedo <= 0.9)).all()


@pytest.mark.slow
def test_large_scene_triangle_budget():
    sc = scenes.large(seed=0)
    assert sc.ntri == 262144  # 4096 boxes x 12 + 64 columns x 3328
    assert sc.dim == 256 and sc.levels == 9 and sc.shadow_size == (2048, 2048) and sc.gbuffer_size == (1920, 1080)
    assert len(sc.lights) == 5 and sc.lights[0]["type"] == 1 and sum(l["type"] == 0 for l in sc.lights) == 4


def test_oracle_thread_count_invariance():
    sc = scenes.tiny(seed=2)
    sm1 = O.render_shadowmap(sc, 1)
    sm4 = O.render_shadowmap(sc, 4)
    assert np.array_equal(sm1, sm4)
    a = O.voxelize(sc, sm1, nthreads=1)
    b = O.voxelize(sc, sm1, nthreads=4)
    assert all(np.array_equal(x, y) for x, y in zip(a[:2], b[:2])) and a[2] == b[2]
    r1 = O.frame(sc, nthreads=1)
    r4 = O.frame(sc, nthreads=4)
    for k in ("color", "normal", "chain", "irradiance", "specular", "out"):
        assert np.array_equal(r1[k], r4[k]), k
    assert r1["stats"] == r4["stats"]


def test_oracle_trace_fp32_close_to_fp64():
    sc = scenes.tiny(seed=5)
    r = O.frame(sc)
    irr64, spec64, _, _ = O.trace(sc, r["chain"], r["gpos"], r["gnrm"], r["galb"], precision=64,
                                  want=("irr", "spec"))
    a = r["irradiance"].reshape(-1, 4)[:, :3].astype(np.float64)
    b = irr64.reshape(-1, 4)[:, :3]
    assert np.linalg.norm(a - b) <= 1e-5 * max(np.linalg.norm(b), 1e-30)


def test_accumulators_are_order_independent():
    sc = scenes.tiny(seed=6)
    sm = O.render_shadowmap(sc)
    a = O.voxelize(sc, sm)
    perm = np.random.default_rng(1).permutation(sc.ntri)
    b = O.voxelize(sc, sm, positions=sc.positions[perm], normals=sc.normals[perm], albedo=sc.albedo[perm])
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]
