"""The tensor-core block passes, planned by the library and executed by a host
functional model of the kernels' data movement (tests/block_model.cpp: the
destination tables, the matrix images with their variants, the staging
slots), compared with the oracle.  CPU only: it checks the planner's grouping,
column and row orders, images and tables for both operand formats, and the
complex128 digit kernel's arithmetic step by step."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

ROOT = Path(__file__).resolve().parent.parent
CUDA_INC = Path("/usr/local/cuda/include")


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    if shutil.which("g++") is None or not CUDA_INC.exists():
        pytest.skip("needs g++ and the CUDA headers")
    from code_mojo_gb300 import build
    lib = build.build_engine()
    exe = tmp_path_factory.mktemp("block_model") / "block_model"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(CUDA_INC), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "block_model.cpp"), "-o", str(exe), "-L", str(lib.parent), "-lbfgpu",
                    f"-Wl,-rpath,{lib.parent}"], check=True, capture_output=True)
    return exe


def run_model(exe, fmt, qc, re, im, tmp_path, shift=None, tiles=False):
    import os
    ops, sin, sout = tmp_path / "ops.bin", tmp_path / "in.bin", tmp_path / "out.bin"
    ops.write_bytes(bfy.serialize(qc))
    (re + 1j * im).astype(np.complex128).tofile(sin)
    env = dict(os.environ)
    env.pop("BFGPU_DIGIT_SCALE_SHIFT", None)
    env.pop("BFGPU_DIGIT_FIVE", None)
    if shift is not None:
        env["BFGPU_DIGIT_SCALE_SHIFT"] = str(shift)
    r = subprocess.run([str(exe), fmt, str(ops), str(sin), str(sout)], check=True, capture_output=True, text=True,
                       env=env)
    fields = [int(x) for x in r.stdout.split()]
    out = np.fromfile(sout, dtype=np.complex128)
    if tiles:
        return out, fields[0], (fields[3], fields[4])
    return out, fields[0]


def random_controlled_circuit(n, count, seed):
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


def gates_only(qc):
    """The circuit without its permutations (the model covers gate circuits)."""
    out = bfy.QuantumCircuit(qc.num_qubits)
    out.transformations = [t for t in qc.transformations if isinstance(t, bfy.GateTransformation)]
    return out


CIRCUITS = {
    "layered13": lambda: W.random_layered_circuit(13, 10, seed=1),
    "layered14": lambda: W.random_layered_circuit(14, 16, seed=2),
    "controlled14": lambda: random_controlled_circuit(14, 160, 3),
    "layered16x40": lambda: W.random_layered_circuit(16, 40, seed=4),
    "qft13": lambda: gates_only(W.qft_circuit(13)),
}


@pytest.mark.parametrize("name", ["layered13", "layered14", "controlled14", "qft13"])
def test_digit_arithmetic_matches_the_oracle(model, name, tmp_path):
    """The digit kernel's own arithmetic (48-bit fixed point relative to the
    scale, exact level sums, carries rounding half to even) stays within
    1e-12 of the oracle and within 5e-13 of the same plan in FP64 (one
    rounding of at most 2^-49 of the scale per block)."""
    qc = CIRCUITS[name]()
    re, im = W.random_normal_state(qc.num_qubits, 7)
    exact, _ = run_model(model, "digits-exact", qc, re, im, tmp_path)
    fp64, _ = run_model(model, "digits", qc, re, im, tmp_path)
    r, i = O.run(qc, re, im)
    assert float(np.max(np.abs(exact - (r + 1j * i)))) <= 1e-12
    assert float(np.max(np.abs(exact - fp64))) <= 5e-13


def test_digit_arithmetic_scales_with_the_norm(model, tmp_path):
    """A state of norm 37: the scale follows it, the error stays 1e-12 relative."""
    qc = CIRCUITS["layered13"]()
    re, im = W.random_normal_state(13, 9)
    got, _ = run_model(model, "digits-exact", qc, 37 * re, 37 * im, tmp_path)
    r, i = O.run(qc, 37 * re, 37 * im)
    assert float(np.max(np.abs(got - (r + 1j * i)))) <= 37e-12


@pytest.mark.parametrize("fmt", ["digits", "tf32"])
@pytest.mark.parametrize("name", list(CIRCUITS))
def test_block_passes_match_the_oracle(model, fmt, name, tmp_path):
    qc = CIRCUITS[name]()
    n = qc.num_qubits
    re, im = W.random_normal_state(n, 7)
    got, block_passes = run_model(model, fmt, qc, re, im, tmp_path)
    r, i = O.run(qc, re, im)
    err = float(np.max(np.abs(got - (r + 1j * i))))
    if name != "qft13":
        assert block_passes > 0
    # digit images hold the matrices to 48 bits; TF32 hi + lo parts to about 2^-22
    assert err <= (1e-12 if fmt == "digits" else 1e-5), err


@pytest.mark.parametrize("shift,tol", [(10, 5e-9), (6, 1e-10)])
def test_five_digit_tiles_match_the_oracle(model, shift, tol, tmp_path):
    """Tiles in five digits: with the scale raised by 2^10 (a unit of
    2^-38 of the norm) every tile of a 14-qubit state falls below 2^-9 of
    it; with 2^6 the tiles of a 16-qubit state (a quarter of the norm each)
    do.  The error follows the coarser unit."""
    qc = CIRCUITS["layered16x40"]() if shift == 6 else CIRCUITS["layered14"]()
    n = qc.num_qubits
    re, im = W.random_normal_state(n, 7)
    got, _, (five, six) = run_model(model, "digits-exact", qc, re, im, tmp_path, shift=shift, tiles=True)
    assert five > 0 and six == 0
    r, i = O.run(qc, re, im)
    assert float(np.max(np.abs(got - (r + 1j * i)))) <= tol


def test_default_scale_keeps_six_digits_on_small_states(model, tmp_path):
    """At 13 qubits a tile holds half the state's norm, far above 2^-9 of
    the scale, so every tile keeps six digits."""
    qc = CIRCUITS["layered13"]()
    re, im = W.random_normal_state(13, 7)
    _, _, (five, six) = run_model(model, "digits-exact", qc, re, im, tmp_path, tiles=True)
    assert five == 0 and six > 0


def test_tiles_below_the_bound_run_five_digits_at_the_state_unit(model, tmp_path):
    """A 16-qubit state whose norm sits almost entirely on qubit 15 = 0: the
    passes' tiles on the other half hold far less than 2^-9 of the scale and
    run five digits, at the same unit as the six-digit tiles, so the result
    stays within 1e-12 of the oracle."""
    n = 16
    qc = W.random_layered_circuit(n, 2, seed=5)
    re, im = W.random_normal_state(n, 8)
    re[1 << 15:] *= 1e-4
    im[1 << 15:] *= 1e-4
    s = np.sqrt(np.sum(re * re + im * im))
    re, im = re / s, im / s
    got, _, (five, six) = run_model(model, "digits-exact", qc, re, im, tmp_path, tiles=True)
    r, i = O.run(qc, re, im)
    assert float(np.max(np.abs(got - (r + 1j * i)))) <= 1e-12
    assert five > 0 and six > 0


def test_five_digit_round_trip_keeps_the_norm(model, tmp_path):
    """Five-digit tiles (scale raised by 2^6 at 16 qubits): the circuit
    followed by its adjoint keeps the norm and returns the state; the load
    of a value that a digit pass wrote is exact, and the first pass's
    rounding of the input ties to even."""
    from code_mojo_gb300 import opsarray as OA
    n = 16
    fwd = W.random_layered_circuit(n, 12, seed=6)
    inv = bfy.QuantumCircuit(n)
    for tr in reversed(fwd.transformations):
        g = tr.gate_info
        inv.add(tr.controls, tr.target, bfy.Custom_Gate(g.gate.conj().T) if g.kind == bfy.GateKind.CUSTOM else g)
    qc = bfy.QuantumCircuit(n)
    qc.transformations = fwd.transformations + inv.transformations
    re, im = W.random_normal_state(n, 3)
    got, _, (five, six) = run_model(model, "digits-exact", qc, re, im, tmp_path, shift=6, tiles=True)
    assert five > 0
    assert abs(float(np.sum(np.abs(got) ** 2)) - 1.0) <= 1e-11
    assert float(np.max(np.abs(got - (re + 1j * im)))) <= 2e-10
    del OA


def random_unitary(dim, rng):
    a = rng.normal(size=(dim, dim)) + 1j * rng.normal(size=(dim, dim))
    q, r = np.linalg.qr(a)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def unitary_circuit(n, count, seed):
    """Gates mixed with dense 2- to 5-qubit unitaries, some controlled."""
    rng = np.random.Generator(np.random.PCG64(seed))
    qc = bfy.QuantumCircuit(n)
    for _ in range(count):
        kind = int(rng.integers(0, 6))
        if kind <= 1 or kind >= 4:
            m = 2 + kind if kind <= 1 else kind  # 2, 3, 4 or 5 qubits
            t = int(rng.integers(0, n - m + 1))
            qc.unitary(random_unitary(1 << m, rng), t, m)
        elif kind == 2:
            m = 2
            t = int(rng.integers(0, n - m + 1))
            c = int(rng.choice([q for q in range(n) if q < t or q >= t + m]))
            qc.c_unitary(random_unitary(4, rng), c, t, m)
        else:
            qs = [int(x) for x in rng.permutation(n)[:2]]
            qc.u3(qs[0], float(rng.uniform(0, 6)), float(rng.uniform(0, 6)), float(rng.uniform(0, 6)))
            qc.cx(qs[0], qs[1])
    return qc


UNITARY_CIRCUITS = {
    "fused_layered14": lambda: __import__("code_mojo_gb300.fusion", fromlist=["fuse_circuit"]).fuse_circuit(
        W.random_layered_circuit(14, 12, seed=5)),
    "unitaries13": lambda: unitary_circuit(13, 60, 6),
}


@pytest.mark.parametrize("fmt", ["digits", "tf32", "digits-exact"])
@pytest.mark.parametrize("name", list(UNITARY_CIRCUITS))
def test_dense_unitaries_in_block_passes(model, fmt, name, tmp_path):
    """Dense 2- to 5-qubit unitaries (from the fusion rewrites, or written
    directly, some controlled) are multiplied into the tensor-core blocks of
    the fused run around them."""
    qc = UNITARY_CIRCUITS[name]()
    assert any(isinstance(t, (bfy.UnitaryTransformation, bfy.ControlledUnitaryTransformation))
               for t in qc.transformations)
    re, im = W.random_normal_state(qc.num_qubits, 11)
    got, block_passes = run_model(model, fmt, qc, re, im, tmp_path)
    r, i = O.run(qc, re, im)
    tol = 1e-12 if fmt.startswith("digits") else 1e-5
    assert block_passes > 0
    assert float(np.max(np.abs(got - (r + 1j * i)))) <= tol


@pytest.mark.parametrize("seed", [31, 32, 33, 34])
@pytest.mark.parametrize("fmt", ["digits", "tf32"])
def test_random_unitary_circuits_in_block_passes(model, fmt, seed, tmp_path):
    """Seeded mixes of gates and 2- to 5-qubit unitaries (some controlled) on
    13 qubits: every plan's grouping and matrices match the oracle."""
    qc = unitary_circuit(13, 40, seed)
    re, im = W.random_normal_state(13, seed)
    got, _ = run_model(model, fmt, qc, re, im, tmp_path)
    r, i = O.run(qc, re, im)
    assert float(np.max(np.abs(got - (r + 1j * i)))) <= (1e-12 if fmt == "digits" else 1e-5)
