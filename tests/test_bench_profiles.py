"""The committed ncu summaries that bench.py reads its roofline figures from
parse, and hold every key the bench line uses."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_flux_update_summary_has_the_roofline_keys():
    prof = bench.ncu_summary("shock_bubble")
    for key in ("profiled_step", "duration_ms", "traffic_bytes_per_launch_full_size", "algorithmic_bytes_per_launch",
                "fp64_flops_per_cell", "fp64_lane_instructions_per_cell", "fp64_pipe_active_frac"):
        assert key in prof and prof[key] > 0, key
    # flops count each fused multiply-add twice, lane instructions once
    assert prof["fp64_flops_per_cell"] >= prof["fp64_lane_instructions_per_cell"]
    assert 0.0 < prof["fp64_pipe_active_frac"] <= 1.0
    assert prof["algorithmic_bytes_per_launch"] == bench.FLUX_BYTES_PER_CELL * 1000 * 400


def test_whole_step_summary_has_the_step_keys():
    step = bench.step_summary("shock_bubble")
    for key in ("profiled_step", "fp64_flops_per_cell_step", "dram_bytes_per_step_cold"):
        assert key in step and step[key] > 0, key
    assert step["fp64_flops_per_cell_step"] > bench.ncu_summary("shock_bubble")["fp64_flops_per_cell"]
