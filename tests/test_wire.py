"""Circuit wire formats: the QASM3 subset of parse_qasm3_string
(utils/qasm3_import.mojo) and the binary op list, on the CPU; a QASM circuit
and a serialized served request on the GPU."""
from __future__ import annotations

import math

import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import opsarray as OA
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

QFT3 = """OPENQASM 3.0;
include "stdgates.inc";
// three-qubit QFT
qubit[3] q;
h q[2];
cp(pi/2) q[1], q[2];
cp(pi/4) q[0], q[2];
h q[1];
cp(pi/2) q[0], q[1];
h q[0];
x q[1];
p(-pi) q[0];
p(0.25*pi) q[1];
p(3/pi) q[2];
p(-1.5) q[0];
"""


def gate_list(qc):
    out = []
    for tr in qc.transformations:
        gi = tr.gate_info
        out.append((int(gi.kind), list(tr.controls), tr.target, float(gi.arg or 0.0)))
    return out


def test_qasm_subset_parses_like_the_reference():
    qc = bfy.parse_qasm3_string(QFT3)
    assert qc.num_qubits == 3
    pi = math.pi
    assert gate_list(qc) == [
        (int(bfy.GateKind.H), [], 2, 0.0), (int(bfy.GateKind.P), [1], 2, pi / 2), (int(bfy.GateKind.P), [0], 2, pi / 4),
        (int(bfy.GateKind.H), [], 1, 0.0), (int(bfy.GateKind.P), [0], 1, pi / 2), (int(bfy.GateKind.H), [], 0, 0.0),
        (int(bfy.GateKind.X), [], 1, 0.0), (int(bfy.GateKind.P), [], 0, -pi), (int(bfy.GateKind.P), [], 1, 0.25 * pi),
        (int(bfy.GateKind.P), [], 2, 3 / pi), (int(bfy.GateKind.P), [], 0, -1.5)]


@pytest.mark.parametrize("text,msg", [
    ("h q[0];", "QASM missing qubit declaration before gates."),
    ("OPENQASM 3.0;\n", "No qubit declaration found in QASM."),
    ("qubit[2] q;\ny q[0];", "Unsupported QASM line: y q[0]"),
    ("qubit[2] q;\nh q0;", "Invalid qubit token: q0"),
    ("qubit[2] q;\ncp(pi) q[0];", "Invalid cp operands: q[0]"),
    ("qubit q;", "Invalid qubit declaration: qubit q;"),
    ("qubit[2] q;\np(2*pi/3) q[0];", "Invalid number in QASM: p(2*pi/3) q[0]"),
])
def test_qasm_errors(text, msg):
    with pytest.raises(F.BFError) as e:
        bfy.parse_qasm3_string(text)
    assert msg in str(e.value)


def test_qasm_circuit_matches_the_circuit_api():
    """The QASM QFT runs bit-identically to the same gates built through the
    circuit API (oracle)."""
    qc = bfy.parse_qasm3_string(QFT3.split("x q[1];")[0])
    ref = bfy.QuantumCircuit(3)
    ref.h(2)
    ref.cp(1, 2, math.pi / 2)
    ref.cp(0, 2, math.pi / 4)
    ref.h(1)
    ref.cp(0, 1, math.pi / 2)
    ref.h(0)
    re, im = W.random_normal_state(3, 4)
    a = O.run(qc, re, im)
    b = O.run(ref, re, im)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def circuit_with_everything(n=6):
    qc = bfy.QuantumCircuit(n)
    qc.h(0)
    qc.cp(0, 3, 0.3)
    qc.add([1, 2], 4, bfy.X_Gate)
    qc.u3(5, 0.1, 0.2, 0.3)
    qc.swap(1, 4)
    qc.qubit_reversal([0, 2, 5])
    u = np.linalg.qr(np.random.default_rng(1).standard_normal((4, 4)) +
                     1j * np.random.default_rng(2).standard_normal((4, 4)))[0]
    qc.unitary(u, 2, 2)
    bfy.bit_reverse(qc, [1, 3, 4])
    bfy.permute_qubits(qc, [5, 4, 3, 2, 1, 0])
    bfy.grover_diffuser(qc, [0, 1, 2])
    bfy.grover_inversion_0(qc)
    bfy.measure(qc, [0, 2], [True, None], seed=7)
    return qc


def test_serialize_round_trip_keeps_every_field():
    qc = circuit_with_everything()
    blob = bfy.serialize(qc)
    assert blob[:4] == b"BFOP"
    back = bfy.deserialize(blob)
    assert back.num_qubits == 6 and len(back) == len(qc.to_ops()[0][:qc.to_ops()[1]])
    a, n, keep = qc.to_ops()
    b, m, keep2 = back.to_ops()
    assert n == m
    for i in range(n):
        x, y = a[i], b[i]
        for f in ("kind", "gate", "target", "target2", "controls", "ncontrols", "flags", "arg", "nqubits"):
            assert getattr(x, f) == getattr(y, f), (i, f)
        assert list(x.mat) == list(y.mat)
        if x.qubits:
            assert [x.qubits[k] for k in range(x.nqubits)] == [y.qubits[k] for k in range(y.nqubits)]
        if x.kind == F.BF_OP_UNITARY:
            d = 2 * (1 << (2 * x.target2))
            assert [x.data[k] for k in range(d)] == [y.data[k] for k in range(d)]
    # a second round gives the same bytes
    assert bfy.serialize(back) == blob
    # the deserialised list runs like the original on the oracle
    re, im = W.random_normal_state(6, 3)
    r1, i1 = O.run(qc, re, im)
    r2, i2 = O.run(back, re, im)
    assert np.array_equal(r1, r2) and np.array_equal(i1, i2)


def test_op_array_circuits_serialise():
    ops = OA.grover(8, 77, iterations=3)
    back = bfy.deserialize(bfy.serialize(ops))
    assert len(back) == len(ops) and back.num_qubits == 8


@pytest.mark.parametrize("mutate,msg", [
    (lambda b: b"XXXX" + b[4:], "not a bfgpu op list"),
    (lambda b: b[:4] + b"\x02\x00\x00\x00" + b[8:], "version 2"),
    (lambda b: b[:-3], "truncated"),
    (lambda b: b + b"\x00" * 8, "trailing bytes"),
    (lambda b: b[:16] + (10 ** 9).to_bytes(8, "little") + b[24:], "count"),
])
def test_corrupt_op_lists_are_refused(mutate, msg):
    blob = bfy.serialize(circuit_with_everything())
    with pytest.raises(F.BFError) as e:
        bfy.deserialize(mutate(blob))
    assert msg in str(e.value)


@pytest.mark.gpu
def test_qasm_circuit_on_the_gpu():
    text = "qubit[12] q;\n" + "".join(f"h q[{i}];\n" for i in range(12)) + \
        "".join(f"cp(pi/{2 ** (k % 5)}) q[{k % 12}], q[{(k * 7 + 3) % 12}];\n" for k in range(40)
                if k % 12 != (k * 7 + 3) % 12)
    qc = bfy.parse_qasm3_string(text)
    re, im = W.random_normal_state(12, 9)
    st = bfy.QuantumState.from_soa(re, im)
    bfy.execute(st, qc)
    got = st.to_complex()
    st.close()
    r, i = O.run(qc, re, im)
    assert np.max(np.abs(got - (r + 1j * i))) <= 1e-12


@pytest.mark.gpu
def test_serialized_request_serves_like_the_direct_one():
    from code_mojo_gb300 import serving as SV
    ops = OA.random_layered(12, 10, 5)
    srv = SV.Server(slots=2)
    a = srv.submit(ops, "c128")
    b = srv.submit_serialized(bfy.serialize(ops), "c128")
    assert srv.wait_idle(60)
    res = {r.id: r for r in srv.poll()}
    srv.close()
    assert res[a].status == 0 and res[b].status == 0
    assert np.array_equal(res[a].top_index, res[b].top_index)
    assert np.array_equal(res[a].top_prob, res[b].top_prob)


def test_random_corruptions_never_crash_the_reader():
    """Byte flips, truncations and spliced counts in a valid op list: the
    reader returns an op list or an error, never reads out of bounds (a
    crash would end this process)."""
    blob = bytearray(bfy.serialize(circuit_with_everything()))
    rng = np.random.Generator(np.random.PCG64(17))
    refused = accepted = 0
    for trial in range(3000):
        b = bytearray(blob)
        kind = trial % 3
        if kind == 0:
            for _ in range(int(rng.integers(1, 8))):
                b[int(rng.integers(0, len(b)))] = int(rng.integers(0, 256))
        elif kind == 1:
            b = b[: int(rng.integers(0, len(b)))]
        else:
            at = int(rng.integers(8, len(b) - 8))
            b[at:at + 8] = int(rng.integers(0, 2 ** 63)).to_bytes(8, "little")
        try:
            back = bfy.deserialize(bytes(b))
            accepted += 1
            assert 1 <= back.num_qubits <= 64
            back.close()
        except F.BFError:
            refused += 1
    assert refused > 0


def test_random_qasm_text_never_crashes_the_parser():
    """Mutated QASM text: parsed or refused with a message, never a crash."""
    base = ("OPENQASM 3.0;\ninclude \"stdgates.inc\";\nqubit[5] q;\nh q[0];\nx q[3];\n"
            "p(pi/4) q[1];\ncp(-pi/8) q[2], q[4];\nh q[4];\n")
    rng = np.random.Generator(np.random.PCG64(23))
    alphabet = "qhxpc[](),;/*-+.0123456789pi \n"
    parsed = 0
    for trial in range(3000):
        t = list(base)
        for _ in range(int(rng.integers(1, 6))):
            at = int(rng.integers(0, len(t)))
            op = int(rng.integers(0, 3))
            if op == 0:
                t[at] = alphabet[int(rng.integers(0, len(alphabet)))]
            elif op == 1:
                del t[at]
            else:
                t.insert(at, alphabet[int(rng.integers(0, len(alphabet)))])
        try:
            qc = bfy.parse_qasm3_string("".join(t))
            parsed += 1
            assert qc.num_qubits >= 1
        except (F.BFError, ValueError):
            pass
    assert parsed > 0
