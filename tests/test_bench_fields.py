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
    assert r["kernel"] == "bf::k_tile<bf::PolDF, false>" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(2 * S / (4200.0 / 74 * 1e-3) / 1e9)
    assert r["traffic"] == pytest.approx(bench.TILE_TRAFFIC_BYTES_PER_AMP * 2 ** n)


def test_digit_flops_per_amplitude_and_block(bench):
    # 26 digit pairs x 2 flops x a 128 x 64 x 64 product per 4096-amplitude tile
    assert bench.DIGIT_FLOPS_PER_AMP_BLOCK == 26 * 2 * 128 * 64 * 64 / 4096 == 6656


def test_per_gate_bytes_of_the_layered_circuit_from_the_gates_alone(bench):
    from code_mojo_gb300 import workloads as W
    # 40 layers x (30 U3 at 2S + 15 CX at S)
    assert bench.per_gate_bytes_in_S(W.random_layered_circuit(30, 40, 0)) == 3000.0
    # QFT-20: 20 H (2S) + 190 CP (S/2), and the bit reversal (2S)
    assert bench.per_gate_bytes_in_S(W.qft_circuit(20, with_bit_reversal=False)) == 20 * 2 + 190 * 0.5
    assert bench.per_gate_bytes_in_S(W.qft_circuit(20)) == 20 * 2 + 190 * 0.5 + 2


def test_hbm_figure_of_the_fused_step(bench):
    plan = {"tile_passes": 51, "block_passes": 50, "blocks": 124, "gate_kernels": 0, "other_passes": 2,
            "bytes_in_S": 104.0}
    h = bench.hbm_figure(plan, 30, 1547.0, 1)
    S = 16.0 * 2 ** 30
    assert h["fused_bytes_per_step"] == 104 * S
    assert h["achieved_GBps"] == pytest.approx(104 * S / 1.547 / 1e9)
    assert h["frac_of_peak"] == pytest.approx(h["achieved_GBps"] / h["peak_GBps"])
    assert h["target_met"] is False


def test_reference_arm_never_loads_the_engine(tmp_path):
    # the reference arm times the oracle's port alone: run it on a small
    # circuit in a child process and look at the libraries it mapped
    import json
    import subprocess
    import sys
    code = (
        "import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--qubits', '14', '--layers', '2', "
        "'--steps', '1', '--warmup', '0']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('ENGINE_MAPPED' if 'libbfgpu' in maps else 'ENGINE_ABSENT')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "ENGINE_ABSENT", r.stdout
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["config"]["qubits"] == 14
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_digit_roofline_counts_five_digit_tiles_at_20_pairs(bench):
    n, S = 30, 16.0 * 2 ** 30
    plan = {"tile_passes": 51, "block_passes": 50, "blocks": 124, "gate_kernels": 0}
    times = {"block_digits": (150, 4500.0)}
    r6 = bench.roofline_of(times, plan, n, S, (0, 100))
    r5 = bench.roofline_of(times, plan, n, S, (100, 0))
    assert r6["digit_pairs_per_block"] == pytest.approx(26) and r5["digit_pairs_per_block"] == pytest.approx(20)
    assert r5["achieved"] == pytest.approx(r6["achieved"] * 20 / 26)
