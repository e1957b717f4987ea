"""bench.py's targets block: each benchmark target with the figure a run
measured, and whether it is met (host logic only, no GPU)."""
import sys

from conftest import ROOT

sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def line_with(copy_gbs, gather_perm_ratio, batch_ratio):
    line = {"peak_gbs": 6661.0,
            "kernels": [{"kernel": f"copy_exit_warp_{w}B", "gbs": g} for w, g in ((4, copy_gbs), (64, 7100.0))]}
    subs = {"gather": {"reference_gpu": {"ratio": 1.04, "ratio_by_pattern": {"perm": gather_perm_ratio}},
                       "ceiling": {"this_frac_perm_min": 0.99, "this_frac_perm_mean": 1.0}},
            "batch": {"details": {"batched_vs_per_call": batch_ratio}}}
    return line, subs


def test_targets_met_and_not_met():
    t = bench.targets(*line_with(6900.0, 1.02, 1.91))
    assert t["copy_at_85pct_of_hbm_peak_4_64B"]["met"] is True
    assert t["copy_at_85pct_of_hbm_peak_4_64B"]["slowest_kernel_gbs"] == 6900.0
    assert t["random_gather_1p2x_reference"]["met"] is False
    assert t["random_gather_1p2x_reference"]["frac_of_random_block_ceiling_perm"]["this_frac_perm_min"] == 0.99
    assert t["batched_2x_per_call"] == {"ratio": 1.91, "met": False}
    t = bench.targets(*line_with(6700.0, 1.25, 2.02))
    assert t["copy_at_85pct_of_hbm_peak_4_64B"]["met"] is False  # 6700 < 0.85 * 8000
    assert t["random_gather_1p2x_reference"]["met"] is True
    assert t["batched_2x_per_call"]["met"] is True


def test_targets_skip_what_did_not_run():
    line, _ = line_with(6900.0, 1.0, 2.0)
    t = bench.targets(line, {})
    assert set(t) == {"copy_at_85pct_of_hbm_peak_4_64B"}
