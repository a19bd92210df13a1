"""Circuits as numpy arrays of bf_op records (the C layout of include/bfgpu.h).

Building long circuits (a 28-qubit Grover search has about 13 000 iterations)
as Python objects is too slow for a serving load, so the request workloads
are built here directly as arrays: random layered circuits, value encodings
and Grover searches.  Grover uses the reference's classical replacements:
the oracle as classical_oracle (grover.mojo:64-66, negate the marked
amplitude) and the diffuser as apply_grover_diffuser (grover_classical.mojo:
284-326, 2*mean - x).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _ffi as F

BF_OP = np.dtype([
    ("kind", "<i4"), ("gate", "<i4"), ("target", "<i4"), ("target2", "<i4"),
    ("controls", "<u8"), ("ncontrols", "<i4"), ("flags", "<u4"), ("arg", "<f8"),
    ("mat", "<f8", (8,)), ("data", "<u8"), ("qubits", "<u8"), ("nqubits", "<i8"),
])
assert BF_OP.itemsize == C.sizeof(F.bf_op) == 128


class OpArray:
    """A circuit as bf_op records plus the buffers its pointers refer to."""

    def __init__(self, n: int, ops: np.ndarray, keep: list):
        self.num_qubits = n
        self.ops = np.ascontiguousarray(ops)
        self.keep = keep

    def __len__(self) -> int:
        return len(self.ops)

    def ptr(self):
        return self.ops.ctypes.data_as(C.POINTER(F.bf_op))

    def to_ops(self):
        """Same contract as QuantumCircuit.to_ops (used by the oracle loader)."""
        return self.ptr(), len(self.ops), [self]


def _gates(count: int) -> np.ndarray:
    a = np.zeros(count, dtype=BF_OP)
    a["kind"] = F.BF_OP_GATE
    return a


def random_layered(n: int, depth: int, seed: int) -> OpArray:
    """depth layers of U3 on every qubit (angles uniform in [0, 2pi)) and CX on
    a random perfect matching, as CUSTOM 2x2 matrices (gates.mojo:42-54)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pairs = n // 2
    per = n + pairs
    a = _gates(depth * per)
    for layer in range(depth):
        ang = rng.uniform(0.0, 2 * math.pi, size=(n, 3))  # same stream as workloads.random_layered_circuit
        th, ph, la = ang[:, 0], ang[:, 1], ang[:, 2]
        c, s = np.cos(th / 2), np.sin(th / 2)
        blk = a[layer * per: layer * per + n]
        blk["gate"] = F.BF_GATE_CUSTOM
        blk["target"] = np.arange(n)
        m = np.zeros((n, 8))
        m[:, 0] = c
        m[:, 2] = -np.cos(la) * s
        m[:, 3] = -np.sin(la) * s
        m[:, 4] = np.cos(ph) * s
        m[:, 5] = np.sin(ph) * s
        m[:, 6] = np.cos(ph + la) * c
        m[:, 7] = np.sin(ph + la) * c
        blk["mat"] = m
        perm = rng.permutation(n)
        cx = a[layer * per + n: (layer + 1) * per]
        cx["gate"] = F.BF_GATE_X
        cx["target"] = perm[1:2 * pairs:2]
        cx["controls"] = np.left_shift(np.uint64(1), perm[0:2 * pairs:2].astype(np.uint64))
        cx["ncontrols"] = 1
        cx["mat"] = np.array([0, 0, 1, 0, 1, 0, 0, 0], dtype=np.float64)
    return OpArray(n, a, [])


def value_encoding(n: int, v: float) -> OpArray:
    """H on all qubits, P(2*pi*2^j*v/2^n) on qubit j, then the inverse QFT over
    the qubits LSB first without swap (value_encoding_circuit.mojo:5-12)."""
    ops = []
    for j in range(n):
        ops.append((F.BF_GATE_H, j, 0, 0.0))
    for j in range(n):
        ops.append((F.BF_GATE_P, j, 0, 2 * math.pi * (2 ** j) * v / 2 ** n))
    t = list(range(n))
    for j in reversed(range(n)):
        ops.append((F.BF_GATE_H, t[j], 0, 0.0))
        for k in reversed(range(j)):
            ops.append((F.BF_GATE_P, t[k], 1 << t[j], -math.pi / 2 ** (j - k)))
    a = _gates(len(ops))
    arr = np.array(ops, dtype=[("g", "<i4"), ("t", "<i4"), ("c", "<u8"), ("a", "<f8")])
    a["gate"] = arr["g"]
    a["target"] = arr["t"]
    a["controls"] = arr["c"]
    a["ncontrols"] = (arr["c"] != 0).astype(np.int32)
    a["arg"] = arr["a"]
    return OpArray(n, a, [])


def grover(n: int, marked: int, iterations: int | None = None) -> OpArray:
    """H^n, then per iteration the classical oracle on |marked> and the
    classical diffuser over all qubits."""
    it = int(math.floor(math.pi / 4 * math.sqrt(2 ** n))) if iterations is None else iterations
    idx = np.array([float(marked)], dtype=np.float64)
    a = np.zeros(n + 2 * it, dtype=BF_OP)
    a[:n]["kind"] = F.BF_OP_GATE
    a[:n]["gate"] = F.BF_GATE_H
    a[:n]["target"] = np.arange(n)
    body = a[n:]
    body["kind"][0::2] = F.BF_OP_CLASSICAL_ORACLE
    body["data"][0::2] = idx.ctypes.data
    body["nqubits"][0::2] = 1
    body["kind"][1::2] = F.BF_OP_GROVER_DIFFUSER
    return OpArray(n, a, [idx])


def adjoint(ops: OpArray) -> OpArray:
    """The inverse of a circuit of gate records: reversed order, each 2x2
    matrix conjugate-transposed (X and other self-inverse gates unchanged in
    effect; P/RX/RY/RZ angles negated)."""
    a = ops.ops[::-1].copy()
    gates = a["kind"] == F.BF_OP_GATE
    if not np.all(gates):
        raise ValueError("adjoint() takes gate records only")
    custom = a["gate"] == F.BF_GATE_CUSTOM
    m = a["mat"][custom]
    # [[m00, m01], [m10, m11]]^dagger = [[m00*, m10*], [m01*, m11*]]
    out = np.empty_like(m)
    out[:, 0], out[:, 1] = m[:, 0], -m[:, 1]
    out[:, 2], out[:, 3] = m[:, 4], -m[:, 5]
    out[:, 4], out[:, 5] = m[:, 2], -m[:, 3]
    out[:, 6], out[:, 7] = m[:, 6], -m[:, 7]
    a["mat"][custom] = out
    angled = np.isin(a["gate"], [F.BF_GATE_P, F.BF_GATE_RX, F.BF_GATE_RY, F.BF_GATE_RZ])
    a["arg"][angled] = -a["arg"][angled]
    return OpArray(ops.num_qubits, a, list(ops.keep))


def batch_mix(count: int = 4096, seed: int = 7, nmin: int = 8, nmax: int = 20, depth: int = 20) -> list[OpArray]:
    """The batched workload: `count` circuits with qubit counts uniform in
    [nmin, nmax]; even positions are random layered circuits of `depth`
    layers, odd ones value encodings with v uniform in [0, 2^n)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        if i % 2 == 0:
            out.append(random_layered(n, depth, int(rng.integers(0, 2 ** 31))))
        else:
            out.append(value_encoding(n, float(rng.uniform(0, 2 ** n))))
    return out
