"""Host-side arithmetic of bench.py's roofline (no GPU): the flop count of the reference's
benchmark, the HBM side of min(FMA peak, bandwidth x intensity), and the DRAM traffic the
committed ncu summary reports per launch."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402


def test_flops_follow_the_reference_benchmark():
    # 6 flops per rotation and row (benchmark/benchmark.jl:10-11): 16384^2, k = 64
    assert bench.flops_per_step(16384, 16384, 64) == pytest.approx(1.0307e11, rel=1e-4)
    assert bench.flops_per_step(1, 2, 1) == 6.0


def test_hbm_side_of_the_roofline():
    algo = (2.0 * 16384 * 16384 + 2.0 * 16383 * 64) * 8
    fl = bench.flops_per_step(16384, 16384, 64)
    h = bench.hbm_side(algo, fl, 121.3, 1.25)
    assert h["intensity_flop_per_byte"] == pytest.approx(23.9, abs=0.05)
    # the FMA peak is the binding side: bandwidth x intensity is two orders above it
    assert h["roofline_tflops"] == pytest.approx(1.25)
    assert h["bw_x_intensity_tflops"] > 100
    assert h["achieved_gbs"] == pytest.approx(algo / 0.1213 / 1e9, abs=0.06)   # rounded to 0.1


def test_traffic_figure_is_committed_and_plausible():
    t = bench.read_traffic()
    assert t is not None
    algo = (2.0 * 16384 * 16384 + 2.0 * 16383 * 64) * 8
    # Q crosses HBM once each way per pass: no more than the algorithmic bytes plus 10 %
    assert 0.5 * algo <= t <= 1.1 * algo
