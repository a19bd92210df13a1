"""Circuit builders for the benchmarked workloads.

  * iqft_circuit / build_iqft_circuit / encode_value_circuit restate
    butterfly/algos/value_encoding_circuit.mojo:5-29;
  * qft_circuit is iqft_circuit(...).inverse() plus the final bit reversal,
    the 20-qubit QFT workload (H on each qubit, n(n-1)/2 controlled phases
    CP(pi/2^k), then the bit-reversal permutation);
  * random_layered_circuit is the 30-qubit random layered workload: per layer
    a U3(theta, phi, lambda) on every qubit with angles uniform in [0, 2pi)
    and a CX on each pair of a seeded random perfect matching;
  * grover_circuit follows butterfly/algos/grover.mojo:45-94 (oracle as an
    X-conjugated multi-controlled phase, then the diffuser).
All randomness comes from numpy's seeded PCG64 generator.
"""
from __future__ import annotations

import math
from typing import Sequence

import numpy as np

from .butterfly import QuantumCircuit, bit_reverse, grover_diffuser, mod_exp


def iqft_circuit(qc: QuantumCircuit, targets: Sequence[int], swap: bool = False) -> None:
    """value_encoding_circuit.mojo:5-12 (MSB-first inverse QFT)."""
    for j in reversed(range(len(targets))):
        qc.h(targets[j])
        for k in reversed(range(j)):
            qc.cp(targets[j], targets[k], -math.pi / 2 ** (j - k))
    if swap:
        bit_reverse(qc, list(targets))


def build_iqft_circuit(n: int, swap: bool = False) -> QuantumCircuit:
    qc = QuantumCircuit(n)
    iqft_circuit(qc, [n - 1 - j for j in range(n)], swap=swap)
    return qc


def encode_value_circuit(n: int, v: float) -> QuantumCircuit:
    """value_encoding_circuit.mojo:19-29: H on all qubits, P(2*pi*v/2^(j+1))
    on qubit j, then the MSB-first IQFT without swap."""
    qc = QuantumCircuit(n)
    for j in range(n):
        qc.h(j)
    for j in range(n):
        qc.p(j, 2 * math.pi / 2 ** (j + 1) * v)
    iqft_circuit(qc, [n - 1 - j for j in range(n)])
    return qc


def qft_circuit(n: int, with_bit_reversal: bool = True) -> QuantumCircuit:
    """QFT as iqft_circuit(...).inverse() (tests/test_qft_classical.mojo:40-56),
    followed by the full bit reversal."""
    qc = QuantumCircuit(n)
    iqft_circuit(qc, [n - 1 - j for j in range(n)], swap=False)
    q = qc.inverse()
    if with_bit_reversal:
        bit_reverse(q)
    return q


def random_layered_circuit(n: int, layers: int, seed: int = 0) -> QuantumCircuit:
    """Per layer: U3 on every qubit (angles uniform in [0, 2pi)), then CX on a
    random perfect matching (seeded shuffle, paired consecutively)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    qc = QuantumCircuit(n)
    for _ in range(layers):
        ang = rng.uniform(0.0, 2 * math.pi, size=(n, 3))
        for q in range(n):
            qc.u3(q, float(ang[q, 0]), float(ang[q, 1]), float(ang[q, 2]))
        perm = rng.permutation(n)
        for k in range(0, n - 1, 2):
            qc.cx(int(perm[k]), int(perm[k + 1]))
    return qc


def grover_iterations(n: int) -> int:
    return int(math.floor(math.pi / 4 * math.sqrt(2 ** n)))


def grover_circuit(n: int, marked: int, iterations: int | None = None) -> QuantumCircuit:
    """H^n, then `iterations` x (phase oracle for `marked`, diffuser)
    (grover.mojo:45-94): the oracle flips the phase of |marked> with X gates
    around an (n-1)-controlled P(pi); the diffuser is H^n, inversion about
    |0> (X^n, MCP(pi), X^n), H^n."""
    it = grover_iterations(n) if iterations is None else iterations
    qc = QuantumCircuit(n)
    for q in range(n):
        qc.h(q)
    ctrls = list(range(n - 1))
    for _ in range(it):
        flips = [q for q in range(n) if not (marked >> q) & 1]
        for q in flips:
            qc.x(q)
        qc.mcp(ctrls, n - 1, math.pi)
        for q in flips:
            qc.x(q)
        for q in range(n):
            qc.h(q)
        for q in range(n):
            qc.x(q)
        qc.mcp(ctrls, n - 1, math.pi)
        for q in range(n):
            qc.x(q)
        for q in range(n):
            qc.h(q)
    return qc


def grover_circuit_classical(n: int, marked: int, iterations: int | None = None) -> QuantumCircuit:
    """The same search with the diffuser as one classical pass (the
    reference's GROVER_DIFFUSER replacement, quantum_circuit.mojo:300-420):
    H^n, then per iteration the phase oracle (X gates around an
    (n-1)-controlled P(pi)) and the diffuser 2*mean - x over all qubits.  The
    classical diffuser differs from the gate one by a global sign, which no
    probability sees."""
    it = grover_iterations(n) if iterations is None else iterations
    qc = QuantumCircuit(n)
    for q in range(n):
        qc.h(q)
    ctrls = list(range(n - 1))
    flips = [q for q in range(n) if not (marked >> q) & 1]
    for _ in range(it):
        for q in flips:
            qc.x(q)
        qc.mcp(ctrls, n - 1, math.pi)
        for q in flips:
            qc.x(q)
        grover_diffuser(qc)
    return qc


def value_encoding_phase_circuit(n: int, v: float) -> QuantumCircuit:
    """H on all n qubits, P(2*pi*2^j*v/2^n) on qubit j, then the inverse QFT
    over the qubits LSB first without swap (gates only): for an integer v the
    result is the bit-reversed basis state |rev(v)>."""
    qc = QuantumCircuit(n)
    for j in range(n):
        qc.h(j)
    for j in range(n):
        qc.p(j, 2 * math.pi * (2 ** j) * v / 2 ** n)
    iqft_circuit(qc, list(range(n)), swap=False)
    return qc


def batch_workload(count: int = 4096, seed: int = 0, nmin: int = 8, nmax: int = 20,
                   depth: int = 20) -> list[QuantumCircuit]:
    """The batched workload: `count` circuits with qubit counts uniform in
    [nmin, nmax]; even positions are random layered circuits of `depth`
    layers, odd ones value encodings with v uniform in [0, 2^n)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        if i % 2 == 0:
            out.append(random_layered_circuit(n, depth, seed=int(rng.integers(0, 2 ** 31))))
        else:
            out.append(value_encoding_phase_circuit(n, float(rng.uniform(0, 2 ** n))))
    return out


def random_normal_state(n: int, seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Amplitudes with re, im i.i.d. N(0, 1) from a seed, normalised to unit
    norm in FP64 (the QFT workload's initial state)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    re = rng.standard_normal(1 << n)
    im = rng.standard_normal(1 << n)
    s = math.sqrt(float(np.sum(re * re) + np.sum(im * im)))
    return re / s, im / s


def modexp_circuit(n_exp: int, n_value: int, a: int, modulus: int) -> QuantumCircuit:
    """modexp_circuit (algos/shor.mojo:143-167): H on the exponent register
    (qubits 0..n_exp-1), |1> in the value register, then MOD_EXP."""
    qc = QuantumCircuit(n_exp + n_value)
    for i in range(n_exp):
        qc.h(i)
    qc.x(n_exp)
    mod_exp(qc, n_exp, n_value, a, modulus)
    return qc


def order_finding_circuit(n_exp: int, n_value: int, a: int, modulus: int, swap: bool = False) -> QuantumCircuit:
    """order_finding_circuit (algos/shor.mojo:334-380): modexp_circuit, then
    the inverse QFT on the exponent register."""
    qc = modexp_circuit(n_exp, n_value, a, modulus)
    iqft_circuit(qc, [n_exp - 1 - j for j in range(n_exp)], swap=swap)
    return qc
