"""The bench's roofline arithmetic on CPU: algorithmic bytes and FLOP per
stage of the production workload (1936x1216 uint8, n = 33, 128-bit
descriptors, step 0.1), and the search's peak -- the FP8 rate measured on
the GPU when the probe ran, twice the measured bf16 GEMM rate otherwise."""
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402

ROWS, COLS, N = 1216, 1936, 33
STAGES = [0.123, 0.751, 0.756]  # ms: transform, search, sweep
CLK = {"sm_mhz": 2070.0}


@pytest.fixture
def fp8_rate():
    saved = dict(bench.FP8_RATE)
    yield bench.FP8_RATE
    bench.FP8_RATE.clear()
    bench.FP8_RATE.update(saved)


def test_sweep_positions():
    # x = -1, then x += step in float32 while x <= 1
    assert bench.sweep_positions(0.1) == 20
    assert bench.sweep_positions(0.25) == 9
    assert bench.sweep_positions(0.5) == 5


def test_algorithmic_bytes_and_flop(fp8_rate):
    fp8_rate.clear()
    r = bench.stage_rooflines(STAGES, ROWS, COLS, N, CLK)
    px = ROWS * COLS
    tiles = ROWS * ((COLS + 127) // 128) * 128 * 32 * 4  # side 1's FP8 candidate tiles
    assert r["transform"]["algorithmic_bytes"] == 2 * px * N + 2 * px * 16 + tiles
    assert r["search"]["algorithmic_flop"] == 2.0 * ROWS * COLS * COLS * 128
    assert r["agreement"]["algorithmic_bytes"] == 2 * px * N + px * 4 + px * 4 + px * 2
    ag = r["agreement"]["fp32"]
    assert ag["algorithmic_flop"] == pytest.approx(12.0 * 0.806 * px * 20 * N)
    # achieved = algorithmic / event time; frac = achieved / peak
    se = r["search"]
    assert se["achieved"] == pytest.approx(se["algorithmic_flop"] / 0.751e-3 / 1e12, abs=0.1)
    assert se["frac"] == pytest.approx(se["achieved"] / se["peak"], abs=1e-3)


def test_search_peak_falls_back_to_twice_bf16(fp8_rate):
    fp8_rate.clear()
    _, bf16, _ = bench.peaks()
    se = bench.stage_rooflines(STAGES, ROWS, COLS, N, CLK)["search"]
    assert se["peak"] == pytest.approx(2 * bf16, abs=0.1)
    assert "2 x" in se["peak_source"]
    assert "shape_peak" not in se


def test_search_peak_is_the_measured_fp8_rate(fp8_rate):
    fp8_rate.clear()
    fp8_rate.update({128: 4800.0, 256: 4850.0})
    _, bf16, _ = bench.peaks()
    se = bench.stage_rooflines(STAGES, ROWS, COLS, N, CLK)["search"]
    assert se["peak"] == 4850.0
    assert "measured FP8" in se["peak_source"]
    assert se["shape_peak"] == 4800.0
    assert se["frac_of_shape_peak"] == pytest.approx(se["achieved"] / 4800.0, abs=1e-3)
    assert se["peak_2x_bf16"] == pytest.approx(2 * bf16, abs=0.1)


def test_probe_failure_leaves_no_rate(fp8_rate):
    class Failing:
        @staticmethod
        def tc_fp8_rate(n):
            raise RuntimeError("no GPU")
    fp8_rate.clear()
    bench.measure_fp8_rate(Failing)
    assert bench.FP8_RATE == {}
