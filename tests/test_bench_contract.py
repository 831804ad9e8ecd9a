"""bench.py's host-side bookkeeping: the per-format ncu counters that scale the dominant kernel's
traffic, L2 bandwidth and issue rate to a timed launch, and the batch configuration block that the
reference arm shares with the measured arm."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_measured_bounds_scale_each_formats_counters():
    import bench
    clk = {"sm_mhz": 2000.0}
    for fmt in ("quantised", "fp32"):
        c = bench.NCU_PER_RAY[fmt]
        out = bench.measured_bounds(4649742, 10.0, clk, fmt)
        assert abs(out["traffic"] - c["dram_bytes"] * 4649742) <= 1
        assert abs(out["l2"]["achieved_gbs"] - c["l2_bytes"] * 4649742 / 10e-3 / 1e9) < 0.1
        peak = 152 * 4 * 2000e6
        assert out["issue"]["peak_per_s"] == peak
        assert abs(out["issue"]["frac"] - c["warp_inst"] * 4649742 / 10e-3 / peak) < 1e-4
        assert out["counters_from"].startswith("profiles/") and os.path.exists(os.path.join(ROOT, out["counters_from"]))
    assert bench.measured_bounds(100, 1.0, clk, "fp16") == {}


def test_batch_config_block_names_the_autotuned_format_choice():
    import bench
    models = [{"nstrands": 10, "nverts": 5, "width": 4, "height": 2, "spp": 3}]
    blk = bench.batch_config_block(models)
    assert blk["segments"] == 40 and blk["primary_samples"] == 24 and blk["scenes"] == 1
    assert blk["precision"] == bench.BATCH_PRECISION_DESC and "autotuner" in blk["precision"]


def test_rank_views_are_disjoint_and_rank0_keeps_the_workload():
    import math
    import bench
    assert bench.rank_azimuth(0.3, 0, 4) == 0.3
    az = [bench.rank_azimuth(0.3, r, 4) % (2 * math.pi) for r in range(4)]
    assert len({round(a, 9) for a in az}) == 4
    assert abs(bench.rank_azimuth(0.3, 2, 4) - (0.3 + math.pi)) < 1e-12
