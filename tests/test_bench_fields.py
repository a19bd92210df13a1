"""The bench line's derived fields, from synthetic pass timings (CPU)."""
import importlib.util
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_digit_roofline_counts_the_blocks_of_the_timed_passes(bench):
    n, S = 30, 16.0 * 2 ** 30
    plan = {"tile_passes": 51, "block_passes": 50, "blocks": 124, "gate_kernels": 0}
    # three circuits: 150 digit passes and 3 double-float passes
    times = {"block_digits": (150, 4500.0), "tile": (3, 100.0)}
    r = bench.roofline_of(times, plan, n, S)
    assert r["kernel"] == "bf::k_tblock_dg" and r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    flops = bench.DIGIT_FLOPS_PER_AMP_BLOCK * 2 ** n * 124 * 3
    assert r["achieved"] == pytest.approx(flops / 4.5 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["avg_launch_ms"] == pytest.approx(30.0)
    assert r["share_of_step"] == pytest.approx(4500 / 4600)
    assert r["hbm"]["achieved"] == pytest.approx(2 * S / 0.030 / 1e9)
    assert r["traffic"] == pytest.approx(bench.DIGIT_TRAFFIC_BYTES_PER_AMP * 2 ** n)


def test_tile_roofline_without_tensor_blocks(bench):
    n, S = 30, 16.0 * 2 ** 30
    times = {"tile": (74, 4200.0), "gate": (1, 2.0)}
    r = bench.roofline_of(times, {"tile_passes": 74, "block_passes": 0, "blocks": 0}, n, S)
    assert r["kernel"] == "bf::k_tile<bf::PolDF>" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(2 * S / (4200.0 / 74 * 1e-3) / 1e9)
    assert r["traffic"] == pytest.approx(bench.TILE_TRAFFIC_BYTES_PER_AMP * 2 ** n)


def test_digit_flops_per_amplitude_and_block(bench):
    # 26 digit pairs x 2 flops x a 128 x 64 x 64 product per 4096-amplitude tile
    assert bench.DIGIT_FLOPS_PER_AMP_BLOCK == 26 * 2 * 128 * 64 * 64 / 4096 == 6656
