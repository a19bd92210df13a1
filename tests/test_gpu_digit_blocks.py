"""complex128 tile passes as 5-qubit blocks on the tensor cores, in exact
base-256 digits (bf16 digit products summed exactly in FP32): parity with the
FP64 oracle at max|Δamp| <= 1e-12 (scaled by the state's norm), with the
double-float CUDA-core path, states of any norm, circuits that are not
norm-preserving (planned without digit passes), pass timing, and the
host-side plan (CPU)."""
from __future__ import annotations

import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

TOL = 1e-12


def ctx(tensor: bool) -> bfy.ExecContext:
    c = bfy.ExecContext()
    c.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    c.gpu_tensor_blocks = tensor
    return c


def run(qc, re, im, tensor=True):
    st = bfy.QuantumState.from_soa(re, im, "c128")
    bfy.execute(st, qc, ctx(tensor))
    out = st.to_complex()
    st.close()
    return out


def oracle(qc, re, im):
    r, i = O.run(qc, re, im)
    return r + 1j * i


def random_controlled_circuit(n, count, seed):
    """CX / CCX / CP / CRY / U3 with controls and targets anywhere."""
    rng = np.random.Generator(np.random.PCG64(seed))
    qc = bfy.QuantumCircuit(n)
    for _ in range(count):
        kind = int(rng.integers(0, 5))
        qs = [int(x) for x in rng.permutation(n)[:3]]
        a = float(rng.uniform(0, 2 * np.pi))
        if kind == 0:
            qc.cx(qs[0], qs[1])
        elif kind == 1:
            qc.ccx(qs[0], qs[1], qs[2])
        elif kind == 2:
            qc.cp(qs[0], qs[1], a)
        elif kind == 3:
            qc.cry(qs[0], qs[1], a)
        else:
            qc.u3(qs[0], a, float(rng.uniform(0, 6)), float(rng.uniform(0, 6)))
    return qc


def test_plan_uses_digit_passes_for_complex128():
    qc = W.random_layered_circuit(16, 8, seed=1)
    on = bfy.plan_stats(qc, ctx(True), "c128")
    off = bfy.plan_stats(qc, ctx(False), "c128")
    assert on["block_passes"] > 0 and off["block_passes"] == 0
    assert on["bytes_in_S"] <= off["bytes_in_S"]


def test_plan_keeps_non_unitary_circuits_off_digit_passes():
    """A gate that changes the norm: the digit scale could not bound the
    state, so the whole circuit stays on double-float passes."""
    qc = W.random_layered_circuit(16, 8, seed=1)
    qc.custom(3, np.array([[1.0, 0.0], [0.0, 0.5]], dtype=np.complex128))
    assert bfy.plan_stats(qc, ctx(True), "c128")["block_passes"] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("n", [12, 14, 16])
def test_random_layered_from_basis(n):
    qc = W.random_layered_circuit(n, 10, seed=n)
    re, im = O.basis(n)
    assert bfy.plan_stats(qc, ctx(True))["block_passes"] > 0
    assert np.max(np.abs(run(qc, re, im) - oracle(qc, re, im))) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("n", [13, 15])
def test_qft_from_random_state(n):
    qc = W.qft_circuit(n)
    re, im = W.random_normal_state(n, 7)
    assert np.max(np.abs(run(qc, re, im) - oracle(qc, re, im))) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_controls_and_targets_anywhere(seed):
    n = 14
    qc = random_controlled_circuit(n, 150, seed)
    re, im = W.random_normal_state(n, seed)
    assert np.max(np.abs(run(qc, re, im) - oracle(qc, re, im))) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("scale", [1e-9, 1e-3, 37.0, 3e5])
def test_states_of_any_norm(scale):
    """The digit scale follows the norm: the error stays 1e-12 relative to it."""
    n = 13
    qc = W.random_layered_circuit(n, 8, seed=3)
    re, im = W.random_normal_state(n, 4)
    re, im = re * scale, im * scale
    got = run(qc, re, im)
    assert np.max(np.abs(got - oracle(qc, re, im))) <= TOL * scale


@pytest.mark.gpu
def test_matches_the_double_float_path():
    n = 16
    qc = W.random_layered_circuit(n, 12, seed=9)
    re, im = W.random_normal_state(n, 9)
    assert np.max(np.abs(run(qc, re, im, True) - run(qc, re, im, False))) <= TOL


@pytest.mark.gpu
def test_non_unitary_circuit_runs_on_double_float():
    n = 13
    qc = W.random_layered_circuit(n, 6, seed=2)
    qc.custom(5, np.array([[1.0, 0.0], [0.0, 0.5]], dtype=np.complex128))
    re, im = W.random_normal_state(n, 2)
    assert np.max(np.abs(run(qc, re, im) - oracle(qc, re, im))) <= TOL


@pytest.mark.gpu
def test_repeated_runs_are_bit_identical():
    """Digit sums are exact: the same input gives the same bits."""
    n = 14
    qc = W.random_layered_circuit(n, 6, seed=5)
    re, im = W.random_normal_state(n, 5)
    assert np.array_equal(run(qc, re, im), run(qc, re, im))


@pytest.mark.gpu
def test_pass_timing_counts_the_plan():
    n = 16
    qc = W.random_layered_circuit(n, 8, seed=6)
    plan = bfy.plan_stats(qc, ctx(True))
    st = bfy.QuantumState(n)
    st.pass_timing(True)
    bfy.execute(st, qc, ctx(True))
    bfy.execute(st, qc, ctx(True))
    t = st.pass_times()
    st.pass_timing(False)
    bfy.execute(st, qc, ctx(True))
    after = st.pass_times()
    st.close()
    assert t["block_digits"][0] == 2 * plan["block_passes"]
    assert t.get("tile", (0, 0))[0] == 2 * (plan["tile_passes"] - plan["block_passes"])
    assert all(ms > 0 for _, ms in t.values())
    assert after == {}


@pytest.mark.gpu
def test_30q_layered_round_trip_in_digits():
    """Full size: the 40-layer circuit then its adjoint returns |0> on the
    digit path (complex128, 16 GiB)."""
    from code_mojo_gb300 import opsarray as OA
    n = 30
    ops = OA.random_layered(n, 40, 0)
    assert bfy.plan_stats(ops, ctx(True))["block_passes"] > 0
    st = bfy.QuantumState(n)
    bfy.execute(st, ops, ctx(True))
    bfy.execute(st, OA.adjoint(ops), ctx(True))
    top_idx, top_p = st.topk(1)
    norm = st.norm2()
    st.close()
    assert int(top_idx[0]) == 0 and top_p[0] >= 1 - 1e-10
    assert abs(norm - 1) <= 1e-11


@pytest.mark.gpu
def test_plans_of_growing_size_on_one_state():
    """A state runs a small digit plan, a larger one (its block buffers grow)
    and the small one again: every result matches the oracle."""
    n = 14
    small = W.random_layered_circuit(n, 2, seed=11)
    large = W.random_layered_circuit(n, 24, seed=12)
    re, im = W.random_normal_state(n, 13)
    st = bfy.QuantumState(n)
    for qc in (small, large, small):
        st.upload(re, im)
        bfy.execute(st, qc, ctx(True))
        assert np.max(np.abs(st.to_complex() - oracle(qc, re, im))) <= TOL
    st.close()


@pytest.mark.gpu
def test_plan_cache_tells_circuits_apart():
    """A state keeps its recent plans keyed by the exact op list: circuits that
    differ only in their matrices, or in the data of a unitary, get their own
    plans, and running one again reuses its plan with the right result."""
    n = 13
    a = W.random_layered_circuit(n, 4, seed=21)
    b = W.random_layered_circuit(n, 4, seed=22)  # same shape, other angles
    u1 = np.linalg.qr(np.random.default_rng(1).normal(size=(4, 4)) + 1j * np.random.default_rng(2).normal(size=(4, 4)))[0]
    u2 = np.linalg.qr(np.random.default_rng(3).normal(size=(4, 4)) + 1j * np.random.default_rng(4).normal(size=(4, 4)))[0]
    c1, c2 = bfy.QuantumCircuit(n), bfy.QuantumCircuit(n)
    c1.transformations = list(a.transformations)
    c2.transformations = list(a.transformations)
    c1.unitary(u1, 3, 2)
    c2.unitary(u2, 3, 2)
    re, im = W.random_normal_state(n, 23)
    st = bfy.QuantumState(n)
    for qc in (a, b, c1, c2, a, c2, b, c1):
        st.upload(re, im)
        bfy.execute(st, qc, ctx(True))
        assert np.max(np.abs(st.to_complex() - oracle(qc, re, im))) <= TOL
    st.close()


@pytest.mark.gpu
@pytest.mark.parametrize("shift", [None, 10, 7])
@pytest.mark.parametrize("layers,seed", [(8, 0), (12, 1), (16, 0)])
def test_digit_passes_equal_the_arithmetic_model_bit_for_bit(layers, seed, shift, tmp_path, monkeypatch):
    """The GPU's digit passes give exactly the bits of the host model of the
    digit arithmetic (tests/block_model.cpp, digits-exact): the same scale
    and unit, digit counts per tile, digits, exact level sums and half-even
    carries.  The circuits are planned as block passes only, so no
    double-float pass is involved.  At 13 qubits every tile keeps six
    digits; with the scale raised by 2^10 every tile runs five, and with
    2^7 the tiles run five or six by their norms."""
    import shutil
    import subprocess
    from pathlib import Path

    from code_mojo_gb300 import build

    root = Path(__file__).resolve().parent.parent
    if shutil.which("g++") is None or not Path("/usr/local/cuda/include").exists():
        pytest.skip("needs g++ and the CUDA headers")
    lib = build.build_engine()
    exe = tmp_path / "block_model"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", "/usr/local/cuda/include", "-I", str(root / "include"),
                    str(root / "tests" / "block_model.cpp"), "-o", str(exe), "-L", str(lib.parent), "-lbfgpu",
                    f"-Wl,-rpath,{lib.parent}"], check=True, capture_output=True)
    import os
    n = 13
    qc = W.random_layered_circuit(n, layers, seed=seed)
    plan = bfy.plan_stats(qc, ctx(True))
    assert plan["block_passes"] == plan["tile_passes"] > 0 and plan["gate_kernels"] == 0
    re, im = W.random_normal_state(n, 7)
    # a state whose norm is spread unevenly over the tiles, so that a
    # middle slack gives both digit counts
    re[: 1 << 12] *= 3.0
    im[: 1 << 12] *= 3.0
    (tmp_path / "ops.bin").write_bytes(bfy.serialize(qc))
    (re + 1j * im).astype(np.complex128).tofile(tmp_path / "in.bin")
    env = dict(os.environ)
    env.pop("BFGPU_DIGIT_SCALE_SHIFT", None)
    env.pop("BFGPU_DIGIT_FIVE", None)
    monkeypatch.delenv("BFGPU_DIGIT_FIVE", raising=False)
    if shift is None:
        monkeypatch.delenv("BFGPU_DIGIT_SCALE_SHIFT", raising=False)
    else:
        env["BFGPU_DIGIT_SCALE_SHIFT"] = str(shift)
        monkeypatch.setenv("BFGPU_DIGIT_SCALE_SHIFT", str(shift))
    r = subprocess.run([str(exe), "digits-exact", str(tmp_path / "ops.bin"), str(tmp_path / "in.bin"),
                        str(tmp_path / "out.bin")], check=True, capture_output=True, text=True, env=env)
    five_model, six_model = (int(x) for x in r.stdout.split()[3:5])
    model = np.fromfile(tmp_path / "out.bin", dtype=np.complex128)
    st = bfy.QuantumState.from_soa(re, im)
    st.digit_tiles(reset=True)
    bfy.execute(st, qc, ctx(True))
    got = st.to_complex()
    five, six = st.digit_tiles()
    st.close()
    assert (five, six) == (five_model, six_model)
    if shift is None:
        assert five == 0 and six > 0
    elif shift == 10:
        assert six == 0 and five > 0
    assert np.array_equal(got, model)


@pytest.mark.gpu
def test_five_digit_tiles_give_the_six_digit_bits(monkeypatch):
    """Five-digit tiles hold the same fixed-point integers as six-digit ones
    (their top digit is zero) and keep the same digit pairs, so a 27-qubit
    circuit gives the same bits with five-digit tiles allowed (most tiles
    take them) and forbidden."""
    n = 27
    qc = W.random_layered_circuit(n, 6, seed=3)
    out = {}
    monkeypatch.delenv("BFGPU_DIGIT_SCALE_SHIFT", raising=False)
    for five in ("1", "0"):
        monkeypatch.setenv("BFGPU_DIGIT_FIVE", five)
        st = bfy.QuantumState(n)
        st.digit_tiles(reset=True)
        bfy.execute(st, qc, ctx(True))
        counts = st.digit_tiles()
        blk = 1 << 22
        h = np.empty(1 << n, dtype=np.complex128)
        for off in range(0, 1 << n, blk):
            re = np.empty(blk)
            im = np.empty(blk)
            F.check(F.lib().bf_state_download_range(st.handle, off, blk, re.ctypes.data, im.ctypes.data))
            h[off:off + blk] = re + 1j * im
        st.close()
        out[five] = (counts, h)
    monkeypatch.delenv("BFGPU_DIGIT_FIVE", raising=False)
    assert out["1"][0][0] > 0 and out["0"][0][0] == 0
    assert np.array_equal(out["1"][1], out["0"][1])
