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


def test_autotune_cache_returns_stored_choice_and_timing(tmp_path):
    """A cached choice comes back with its stored timing and no device work; fields a cache
    written by an earlier version lacks keep the base parameters' values."""
    import json
    import vkhrt_gb300 as H
    cache = tmp_path / "tune.json"
    cache.write_text(json.dumps({"k": {"kernel_variant": 3, "refill": 16, "speculative": 1, "split_types": 1,
                                       "leaf_again": 2, "ms": 23.5}}))
    base = H.trace_params(shading=2)
    best, ms = H.autotune(None, [], base, cache=str(cache), key="k")
    assert ms == 23.5
    assert (best.kernel_variant, best.refill, best.split_types, best.leaf_again) == (3, 16, 1, 2)
    assert best.variant_by_type == base.variant_by_type == 0 and best.shading == 2
