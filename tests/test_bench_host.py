"""Host-side pieces of the benchmark's JSON line, without a GPU: the
throttle-reason and clock summary of the nvidia-smi samples (a run that saw
hw_slowdown, hw_thermal_slowdown or sw_thermal_slowdown is rejected, so the
parsing must find them), the algorithmic bytes behind `roofline`, and the
peak denominators."""

from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402
from vct_gb300 import scenes  # noqa: E402

# index, clocks.sm, clocks.max.sm, power.draw, reasons.active, hw_slowdown, hw_thermal_slowdown,
# sw_thermal_slowdown, sw_power_cap (nvidia-smi --format=csv,noheader,nounits)
_IDLE = "0, 2070, 2070, 412.3, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
_CAPPED = "0, 1980, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
_THERMAL = "0, 1500, 2070, 1200.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active"


def _summary(lines):
    c = bench.ClockSampler(0)
    c.lines = list(lines)
    return c.summary()


def test_clock_summary_median_and_reasons():
    s = _summary([_IDLE, _IDLE, _CAPPED])
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    s = _summary([_IDLE, _THERMAL, _THERMAL])
    assert s["sm_mhz"] == 1500.0
    assert s["reasons"] == ["hw_thermal_slowdown"]


def test_clock_summary_ignores_malformed_lines():
    s = _summary(["", "[N/A]", "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active", _IDLE])
    assert s["samples"] == 1 and s["sm_mhz"] == 2070.0 and s["reasons"] == []
    assert _summary([])["sm_mhz"] is None


def test_algorithmic_bytes_of_the_large_frame():
    sc = scenes.large(seed=0)
    # the voxeliser's counters of this scene (seed 0), as the frame reports them
    stats = {"total_voxel_fragments": 6666268, "unique_voxels": 5181082}
    a = bench.algorithmic_bytes(sc, stats, None)
    N, T = 256, 262144
    nv = N ** 3
    assert a["accumulate"] == T * 84 + 5181082 * 64 + nv // 8
    assert a["trace"] == 1920 * 1080 * 64  # every pixel covered unless the counters say otherwise
    a = bench.algorithmic_bytes(sc, dict(stats, covered_pixels=1000), None)
    assert a["trace"] == 1920 * 1080 * 32 + 1000 * 32
    assert a["inject_mark"] == 2048 * 2048 * 4 + nv // 8
    lv = lambda lo, hi: sum((N >> l) ** 3 for l in range(lo, hi))  # noqa: E731
    assert a["resolve"] == nv // 4 + 5181082 * 64 + nv * 24 + lv(1, 5) * 8 + lv(0, 5) * 16
    assert a["mip_tail"] == (N >> 4) ** 3 * 8 + lv(5, 9) * 24
    # 1.06 GB for resolve + tail: 170 MB read (masks, occupied records), 895 MB written
    assert 1.0e9 < a["resolve"] + a["mip_tail"] < 1.1e9
    # the hybrid sampler's fused frame: both sampler copies, the linear chain from level 4 on
    h = bench.algorithmic_bytes(sc, stats, None, sampler="hybrid", fused_single=True)
    assert h["resolve"] == nv // 4 + 5181082 * 64 + nv * 16 + lv(4, 5) * 8 + lv(0, 5) * 24
    assert h["mip_tail"] == (N >> 4) ** 3 * 8 + lv(5, 9) * 32
    # a batch writes the whole linear chain as well
    b = bench.algorithmic_bytes(sc, stats, None, sampler="hybrid")
    assert b["resolve"] - h["resolve"] == lv(0, 4) * 8


def test_peaks_come_from_the_measured_file():
    p = bench.load_peaks()
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        assert p["source"] == "measured" and p["hbm_gbs"] > 1000 and p["bf16_tflops"] > 100
    else:
        assert p["source"] == "fallback" and p["hbm_gbs"] == 6800.0


def test_stage_rooflines():
    alg = {"accumulate": 400e6, "resolve": 1000e6, "mip_tail": 60e6, "trace": 130e6, "inject_mark": 20e6}
    ms = {"accumulate": 0.4, "resolve+mips": 0.25, "trace": 0.6, "inject_mark": 0.002}
    s = bench.stage_rooflines(alg, ms, 6800.0, {"trace": 98e6}, 6_000_000, "raster")
    assert set(s) == {"accumulate", "resolve+mips", "trace"}
    r = s["resolve+mips"]
    assert r["algorithmic_bytes"] == 1060000000 and r["achieved_gbs"] == 4240.0
    assert r["frac"] == round(4240.0 / 6800.0, 4) and r["traffic"] is None
    assert s["trace"]["traffic"] == 98e6
    a = s["accumulate"]
    assert a["fragments_per_s"] == 1.5e10 and a["reductions_per_s"] == 7.5e10
    t = bench.stage_rooflines(alg, ms, 6800.0, {}, 6_000_000, "tess")["accumulate"]
    assert t["reductions_per_s"] == 6.0e10


def test_irradiance_accuracy():
    import numpy as np

    rng = np.random.default_rng(0)
    ref = rng.uniform(0.1, 1.0, size=(1000, 4)).astype(np.float32)
    cov = np.ones(1000, dtype=bool)
    cov[:100] = False
    gpu = ref.copy()
    gpu[100:, :3] *= 1.0005  # every judged pixel off by 5e-4 of its value
    gpu[:100] = 7.0  # uncovered pixels are not judged
    a = bench.irradiance_accuracy(gpu, ref, cov)
    assert a["pixels"] == 900 and a["pixels_judged"] == 900
    assert abs(a["rel_l2"] - 5e-4) < 1e-6 and abs(a["max_rel"] - 5e-4) < 1e-6
    assert a["frac_within_1e-3"] == 1.0
    # a dark pixel below the floor counts in rel_l2 but not in the per-pixel figures
    ref2 = ref.copy()
    ref2[500, :3] = 1e-9
    gpu2 = ref2.copy()
    gpu2[500, :3] = 1e-3
    b = bench.irradiance_accuracy(gpu2, ref2, cov)
    assert b["pixels_judged"] == 899 and b["max_rel"] == 0.0 and b["rel_l2"] > 0.0


def test_cpu_model_names():
    assert bench.cpu_model("processor : 0\nmodel name : Intel(R) Xeon(R) CPU @ 2.70GHz\n") == \
        "Intel(R) Xeon(R) CPU @ 2.70GHz"
    grace = "processor : 0\nCPU implementer : 0x41\nCPU architecture: 8\nCPU part : 0xd4f\n"
    assert bench.cpu_model(grace) == "Neoverse-V2 (Arm part 0xd4f)"
    assert "0x123" in bench.cpu_model("CPU implementer : 0x51\nCPU part : 0x123\n")


def test_ncu_traffic_only_for_the_captured_sources():
    digest = bench.kernel_sources_digest()
    assert len(digest) == 16
    traffic, note = bench.ncu_traffic(False)
    assert traffic == {} and "no ncu capture" in note["traffic_source"]
    saved = bench.NCU_CAPTURE_DIGEST
    try:
        bench.NCU_CAPTURE_DIGEST = digest
        traffic, note = bench.ncu_traffic(True)
        assert traffic == bench.NCU_TRAFFIC and note["traffic_digest"] == digest
        bench.NCU_CAPTURE_DIGEST = "0" * 16
        traffic, note = bench.ncu_traffic(True)
        assert traffic == {} and "traffic_stale" in note
    finally:
        bench.NCU_CAPTURE_DIGEST = saved


def test_both_arms_share_the_config_keys():
    import argparse

    sc = scenes.cornell(seed=0)
    args = argparse.Namespace(config="cornell", voxelizer="raster", warp="none", seed=0)
    ours = bench.frame_config(args, sc, 1)
    assert {"workload", "triangles", "grid", "levels", "shadow_map", "gbuffer", "cones", "voxelizer", "warp",
            "l2"} <= set(ours)


def test_accuracy_block_on_the_oracles_own_frame():
    """The bench's accuracy block judged on the oracle's own fp32 frame: the
    chain matches itself, the fp32 trace is 0 from itself and within the
    1e-3 bar of the fp64 trace."""
    import oracle as O

    sc = scenes.cornell(seed=0)
    sm, gb = O.render_shadowmap(sc), O.render_gbuffer(sc)
    ms, detail, chain, (irr, _, _, _) = bench.cpu_frame(sc, 4, 0, sm, gb, want=("irr", "color"))
    assert ms > 0 and detail["rows_traced"] == sc.gbuffer_size[1]
    art = {"irr": {"software": irr}, "chain": chain, "gbuf": gb, "sm": sm}
    a = bench.accuracy_block(sc, art, chain, irr, "software", 4)
    assert a["chain_bitexact"] and a["meets_bar"]
    s = a["samplers"]["software"]
    assert s["vs_fp32_oracle_rel_l2"] == 0.0 and 0.0 < s["vs_fp64"]["rel_l2"] < 1e-5


def test_pareto_front():
    pts = [{"ms": 1.0, "rel_l2": 0.05}, {"ms": 0.5, "rel_l2": 0.2}, {"ms": 1.2, "rel_l2": 0.06},
           {"ms": 2.0, "rel_l2": 0.01}, {"ms": 0.5, "rel_l2": 0.3}]
    f = bench.pareto_front(pts)
    assert [(p["ms"], p["rel_l2"]) for p in f] == [(0.5, 0.2), (1.0, 0.05), (2.0, 0.01)]
