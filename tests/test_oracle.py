"""Pins the CPU oracle (a restatement of the reference's SCALAR strategy)
against the known answers the reference's own tests hold, and against the
golden fixtures made from numpy's FFT (tests/golden/make_golden.py)."""
import math
from pathlib import Path

import numpy as np
import pytest

from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

GOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "qft_golden.npz")


def cplx(t):
    return t[0] + 1j * t[1]


def split(z):
    return np.ascontiguousarray(z.real), np.ascontiguousarray(z.imag)


# ---- tests/test_qft_classical.mojo: gate QFT/IQFT vs the classical FFT ----
@pytest.mark.parametrize("n", [4, 6, 8])
@pytest.mark.parametrize("seed", [3, 7, 11])
@pytest.mark.parametrize("inverse", [False, True])
@pytest.mark.parametrize("swap", [False, True])
def test_gate_qft_matches_golden_fft(n, seed, inverse, swap):
    key = f"n{n}_s{seed}"
    psi = GOLDEN[key + "_in"]
    expect = GOLDEN[key + ("_iqft" if inverse else "_qft") + ("_swap" if swap else "")]
    qc = bfy.QuantumCircuit(n)
    W.iqft_circuit(qc, [n - 1 - j for j in range(n)], swap=swap)
    if not inverse:
        qc = qc.inverse()
    out = cplx(O.run(qc, *split(psi)))
    assert np.max(np.abs(out - expect)) < 1e-13


@pytest.mark.parametrize("targets", [[3, 2, 1, 0], [3, 1]])
@pytest.mark.parametrize("swap", [False, True])
@pytest.mark.parametrize("seed", [3, 7, 11])
def test_gate_qft_matches_classical_restatement(targets, swap, seed):
    # the reference's exact cases (n=4, targets [3,2,1,0] and [3,1], 1e-5)
    n = 4
    re, im = W.random_normal_state(n, seed)
    for inverse in (False, True):
        qc = bfy.QuantumCircuit(n)
        W.iqft_circuit(qc, targets, swap=swap)
        if not inverse:
            qc = qc.inverse()
        gate = cplx(O.run(qc, re, im))
        classical = cplx(O.qft_classical(re, im, targets, inverse=inverse, swap=swap))
        assert np.max(np.abs(gate - classical)) < 1e-12


def test_classical_qft_matches_numpy():
    n = 6
    z = GOLDEN["n6_s3_in"]
    out = cplx(O.qft_classical(*split(z), [], inverse=False, swap=False))
    # LSB-first full register, swap=False: pre bit reversal then FFT
    idx = np.arange(1 << n)
    rev = np.zeros_like(idx)
    for b in range(n):
        rev |= ((idx >> b) & 1) << (n - 1 - b)
    assert np.max(np.abs(out - np.fft.ifft(z[rev]) * np.sqrt(1 << n))) < 1e-13


# ---- tests/test_bit_reverse.mojo --------------------------------------------
@pytest.mark.parametrize("seed", [5, 11, 17])
def test_full_bit_reverse_matches_partial(seed):
    n = 4
    re, im = W.random_normal_state(n, seed)
    a = bfy.QuantumCircuit(n)
    bfy.bit_reverse(a)
    b = bfy.QuantumCircuit(n)
    bfy.bit_reverse(b, [0, 1, 2, 3])
    ra, rb = O.run(a, re, im), O.run(b, re, im)
    assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])


@pytest.mark.parametrize("seed", [7, 13, 19])
@pytest.mark.parametrize("targets", [[], [0, 1, 2, 3], [1, 3]])
def test_bit_reverse_is_involution(seed, targets):
    n = 4
    re, im = W.random_normal_state(n, seed)
    qc = bfy.QuantumCircuit(n)
    bfy.bit_reverse(qc, targets)
    bfy.bit_reverse(qc, targets)
    out = O.run(qc, re, im)
    assert np.array_equal(out[0], re) and np.array_equal(out[1], im)


def test_bit_reverse_index_map():
    n = 10
    re = np.arange(1 << n, dtype=np.float64)
    im = -re
    qc = bfy.QuantumCircuit(n)
    bfy.bit_reverse(qc)
    out = O.run(qc, re, im)
    rev = O.bit_reverse_indices(n).astype(np.int64)
    assert np.array_equal(out[0], re[rev])


# ---- tests/test_circuit_inverse.mojo: U U^-1 |0> = |0> -----------------------
def _roundtrip(build):
    n = 3
    qc = bfy.QuantumCircuit(n)
    build(qc)
    full = bfy.QuantumCircuit(n)
    full.transformations = qc.transformations + qc.inverse().transformations
    out = cplx(O.run(full, *O.basis(n)))
    expect = np.zeros(1 << n, dtype=complex)
    expect[0] = 1
    assert np.max(np.abs(out - expect)) < 1e-12


def test_inverse_x_h():
    _roundtrip(lambda qc: (qc.x(0), qc.h(1)))


def test_inverse_rx_p():
    _roundtrip(lambda qc: (qc.rx(0, 0.3), qc.p(2, 1.1)))


def test_inverse_h_cx_ry_cp():
    _roundtrip(lambda qc: (qc.h(0), qc.cx(0, 1), qc.ry(2, 0.7), qc.cp(1, 2, 0.4)))


# ---- analytic states ---------------------------------------------------------
@pytest.mark.parametrize("n", [3, 5, 8])
def test_h_all_is_uniform(n):
    qc = bfy.QuantumCircuit(n)
    for q in range(n):
        qc.h(q)
    out = cplx(O.run(qc, *O.basis(n)))
    assert np.max(np.abs(out - GOLDEN[f"hn_{n}"])) < 1e-15


@pytest.mark.parametrize("n,v", [(4, 5), (6, 37), (8, 200)])
def test_value_encoding_of_integer_is_basis_state(n, v):
    out = cplx(O.run(W.encode_value_circuit(n, v), *O.basis(n)))
    expect = np.zeros(1 << n, dtype=complex)
    expect[v] = 1
    assert np.max(np.abs(out - expect)) < 1e-12


def test_grover_finds_marked():
    n, marked = 6, 45
    out = cplx(O.run(W.grover_circuit(n, marked), *O.basis(n)))
    p = np.abs(out) ** 2
    assert int(np.argmax(p)) == marked and p[marked] > 0.9


# ---- the parallel port equals the scalar oracle ------------------------------
# bench_execution_strategies.mojo:173-203 checks every strategy against SCALAR.
@pytest.mark.parametrize("builder", [
    lambda: W.encode_value_circuit(12, 4.7),
    lambda: W.random_layered_circuit(12, 4, seed=2),
    lambda: W.qft_circuit(11),
    lambda: W.grover_circuit(7, 99, iterations=2),
])
def test_parallel_port_matches_scalar(builder):
    qc = builder()
    n = qc.num_qubits
    re, im = W.random_normal_state(n, 1)
    s = cplx(O.run(qc, re, im))
    p = cplx(O.run(qc, re, im, strategy=O.OR_SIMD_PARALLEL, threads=4, chunks=8))
    assert np.max(np.abs(s - p)) <= 1e-12


def test_specialised_and_generic_kernels_agree():
    qc = bfy.QuantumCircuit(8)
    for q in range(8):
        qc.h(q)
        qc.ry(q, 0.3 + q)
        qc.p(q, 0.1 * q)
        qc.x(q)
    for q in range(7):
        qc.cp(q, q + 1, 0.2)
        qc.cx(q + 1, q)
        qc.cry(q, q + 1, 0.9)
    re, im = W.random_normal_state(8, 4)
    a = cplx(O.run(qc, re, im, specialized=127))
    b = cplx(O.run(qc, re, im, specialized=0))
    assert np.max(np.abs(a - b)) < 1e-13


# ---- fused pairs and permutations -------------------------------------------
def test_fused_pairs_match_unfused():
    n = 6
    re, im = W.random_normal_state(n, 8)
    pairs = [
        (bfy.GateTransformation([], 1, bfy.H_Gate), bfy.GateTransformation([], 2, bfy.H_Gate)),
        (bfy.GateTransformation([], 3, bfy.H_Gate), bfy.GateTransformation([], 4, bfy.P_Gate(0.3))),
        (bfy.GateTransformation([], 0, bfy.P_Gate(0.7)), bfy.GateTransformation([], 5, bfy.P_Gate(-1.2))),
        (bfy.GateTransformation([0], 2, bfy.P_Gate(0.5)), bfy.GateTransformation([0], 4, bfy.P_Gate(0.9))),
        (bfy.GateTransformation([], 2, bfy.RY_Gate(0.5)), bfy.GateTransformation([2], 3, bfy.X_Gate)),
    ]
    for a, b in pairs:
        fused = bfy.QuantumCircuit(n)
        fused.append_fused_pair(a, b)
        plain = bfy.QuantumCircuit(n)
        plain.transformations = [a, b]
        x = cplx(O.run(fused, re, im))
        y = cplx(O.run(plain, re, im))
        assert np.max(np.abs(x - y)) < 1e-13


def test_permute_qubits_semantics():
    n = 5
    re = np.arange(1 << n, dtype=np.float64)
    im = np.zeros(1 << n)
    order = [3, 0, 4, 1, 2]
    qc = bfy.QuantumCircuit(n)
    bfy.permute_qubits(qc, order)
    out = O.run(qc, re, im)[0].astype(np.int64)
    # destination bit p takes source bit order[p]
    for j in range(1 << n):
        src = 0
        for p in range(n):
            src |= ((j >> p) & 1) << order[p]
        assert out[j] == src


def test_swap_and_qrev_are_exact_permutations():
    n = 6
    re = np.arange(1 << n, dtype=np.float64)
    im = -re
    qc = bfy.QuantumCircuit(n)
    qc.swap(1, 4)
    qc.qubit_reversal([0, 2, 5])
    out = O.run(qc, re, im)
    assert sorted(out[0].tolist()) == re.tolist()


# ---- validation mirrors validate_circuit (executors.mojo:90-185) -------------
@pytest.mark.parametrize("build,msg", [
    (lambda qc: qc.h(9), "Target out of bounds: 9"),
    (lambda qc: qc.cx(7, 1), "Control out of bounds: 7"),
    (lambda qc: qc.unitary(np.eye(4), 3, 2), "Target range out of bounds"),
    (lambda qc: qc.c_unitary(np.eye(4), 1, 0, 2), "Control overlaps target range"),
])
def test_oracle_validation_messages(build, msg):
    qc = bfy.QuantumCircuit(4)
    build(qc)
    with pytest.raises(O.OracleError, match=msg):
        O.run(qc, *O.basis(4))


# ---- apply_measure (state.mojo:447-553) ---------------------------------------
def test_measure_draw_follows_the_reference_generator():
    n = 6
    re, im = W.random_normal_state(n, 21)
    p = re ** 2 + im ** 2
    for seed in (1, 7, 12345, 2 ** 40 + 3):
        oc, pr, r2, i2 = O.measure(re, im, [0, 1, 2, 3, 4, 5], None, seed)
        rng = (seed % 2147483647) * 48271 % 2147483647
        r = rng / 2147483647 * p.sum()
        assert oc == int(np.searchsorted(np.cumsum(p), r))
        assert abs(pr - p[oc]) < 1e-15
        assert abs(r2[oc] ** 2 + i2[oc] ** 2 - 1) < 1e-12


def test_measure_subset_and_postselection():
    n = 5
    re, im = W.random_normal_state(n, 22)
    oc, pr, r2, i2 = O.measure(re, im, [3, 1], [None, True], 99)
    z = r2 + 1j * i2
    assert abs(np.sum(np.abs(z) ** 2) - 1) < 1e-12
    idx = np.arange(1 << n)
    assert np.all(z[((idx >> 1) & 1) == 0] == 0)
    assert np.all(z[((idx >> 3) & 1) != oc] == 0)


def test_topk_orders_by_probability_then_index():
    re = np.array([0.1, 0.5, 0.5, 0.2, 0.0, 0.3, 0.5, 0.1])
    im = np.zeros(8)
    idx, pr = O.topk(re, im, 4)
    assert idx.tolist() == [1, 2, 6, 5]


def test_measure_op_inside_a_circuit_runs_on_the_oracle():
    n = 6
    qc = W.random_layered_circuit(n, 2, seed=3)
    bfy.measure(qc, [1, 4], seed=5)
    re, im = O.basis(n)
    r, i = O.run(qc, re, im)
    z = r + 1j * i
    assert abs(np.sum(np.abs(z) ** 2) - 1) < 1e-12
    idx = np.arange(1 << n)
    nz = idx[np.abs(z) > 0]
    assert len(set(((nz >> 1) & 1).tolist())) == 1 and len(set(((nz >> 4) & 1).tolist())) == 1


# ---- classical Grover passes (grover_classical.mojo:262-326) ------------------
@pytest.mark.parametrize("targets", [[], [0, 2, 3], [4]])
def test_classical_diffuser_is_minus_the_gate_diffuser(targets):
    n = 5
    re, im = W.random_normal_state(n, 50)
    t = targets or list(range(n))
    gate = bfy.QuantumCircuit(n)
    for q in t:
        gate.h(q)
    for q in t:
        gate.x(q)
    if len(t) > 1:
        gate.mcp(t[:-1], t[-1], math.pi)
    else:
        gate.p(t[0], math.pi)
    for q in t:
        gate.x(q)
    for q in t:
        gate.h(q)
    classical = bfy.QuantumCircuit(n)
    bfy.grover_diffuser(classical, targets)
    a = cplx(O.run(gate, re, im))
    b = cplx(O.run(classical, re, im))
    assert np.max(np.abs(a + b)) < 1e-13


def test_classical_inversion_matches_gates():
    n = 5
    re, im = W.random_normal_state(n, 51)
    t = [1, 3, 4]
    gate = bfy.QuantumCircuit(n)
    for q in t:
        gate.x(q)
    gate.mcp(t[:-1], t[-1], math.pi)
    for q in t:
        gate.x(q)
    classical = bfy.QuantumCircuit(n)
    bfy.grover_inversion_0(classical, t)
    assert np.max(np.abs(cplx(O.run(gate, re, im)) - cplx(O.run(classical, re, im)))) < 1e-15


def test_classical_grover_finds_marked():
    n, marked = 8, 201
    p = np.abs(cplx(O.run(W.grover_circuit_classical(n, marked), *O.basis(n)))) ** 2
    assert int(np.argmax(p)) == marked and p[marked] > 0.99
