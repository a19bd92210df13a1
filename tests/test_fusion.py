"""The circuit fusion rewrites (code_mojo_gb300/fusion.py, restating
butterfly/core/transformations_fusion.mojo) on the CPU: their matrix
conventions, the transformations they produce, and that a fused circuit
gives the unfused circuit's state on the oracle."""
import math

import numpy as np
import pytest

from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import fusion as FU
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

TOL = 1e-12

CX4 = np.array([[1, 0, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0]], dtype=complex)  # control b0, target b1


def kinds(trs):
    return [type(t).__name__ for t in trs]


def test_matrix_conventions():
    # basis index b0 + 2 b1, b0 the bit of q_low
    m = FU.controlled_gate_to_matrix4x4(bfy.X, 4, 4, 5)
    assert np.array_equal(m, CX4)
    # control on the high bit, target on the low bit
    m = FU.controlled_gate_to_matrix4x4(bfy.X, 4, 5, 4)
    assert np.array_equal(m, np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=complex))
    h = bfy.H
    assert np.allclose(FU.gate_to_matrix4x4(h, 2, 2), np.kron(np.eye(2), h))
    assert np.allclose(FU.gate_to_matrix4x4(h, 2, 3), np.kron(h, np.eye(2)))
    # later gates multiply on the left
    assert np.allclose(FU.mul_gate(bfy.X, bfy.H), bfy.X @ bfy.H)


def test_can_fuse_special_pair_cases():
    G = bfy.GateTransformation
    h = lambda t: G([], t, bfy.H_Gate)  # noqa: E731
    p = lambda t, a=0.3: G([], t, bfy.P_Gate(a))  # noqa: E731
    cp = lambda c, t, a=0.3: G([c], t, bfy.P_Gate(a))  # noqa: E731
    assert FU.can_fuse_special_pair(h(3), h(4))
    assert not FU.can_fuse_special_pair(h(3), h(5))     # not adjacent
    assert not FU.can_fuse_special_pair(h(3), h(3))     # one qubit
    assert FU.can_fuse_special_pair(p(7), p(6))
    assert FU.can_fuse_special_pair(h(2), cp(2, 3)) and FU.can_fuse_special_pair(cp(3, 2), h(3))
    assert not FU.can_fuse_special_pair(h(2), cp(2, 4))
    assert FU.can_fuse_special_pair(cp(9, 1), cp(9, 5))  # shared control, any distance
    assert not FU.can_fuse_special_pair(cp(9, 1), cp(9, 1))
    assert not FU.can_fuse_special_pair(h(2), p(3))     # HP is not among the pairs it forms
    assert not FU.can_fuse_special_pair(G([0, 1], 2, bfy.X_Gate), h(2))


def test_same_target_runs():
    qc = bfy.QuantumCircuit(4)
    qc.p(1, 0.25)
    qc.p(1, 0.5)
    qc.p(1, -0.125)      # P run -> P(0.625)
    qc.h(2)
    qc.x(2)              # H then X -> unitary X.H
    qc.cp(0, 3, 0.2)
    qc.cp(0, 3, 0.3)     # controlled P run -> CP(0.5)
    qc.h(1)              # another target: ends the run
    qc.cx(0, 3)
    qc.cp(0, 3, 0.1)     # same target and control: joins, the run is no longer all P
    qc.ccx(0, 1, 2)      # multi-controlled: passes through
    qc.h(1)
    out = FU.fuse_same_target_gates(qc.transformations)
    assert kinds(out) == ["GateTransformation", "UnitaryTransformation", "GateTransformation", "GateTransformation",
                          "ControlledUnitaryTransformation", "GateTransformation", "GateTransformation"]
    assert out[0].gate_info.kind == bfy.GateKind.P and out[0].gate_info.arg == pytest.approx(0.625)
    assert np.allclose(out[1].u.reshape(2, 2), bfy.X @ bfy.H) and out[1].m == 1
    assert out[2].controls == [0] and out[2].gate_info.arg == pytest.approx(0.5)
    assert out[3].target == 1 and out[3].gate_info.kind == bfy.GateKind.H
    assert np.allclose(out[4].u.reshape(2, 2), bfy.P(0.1) @ bfy.X) and out[4].control == 0
    assert out[5].controls == [0, 1]


def test_specialized_pairs_of_the_value_encoding_circuit():
    qc = FU.fuse_circuit_specialized_pairs(W.encode_value_circuit(6, 4.7))
    k = kinds(qc.transformations)
    # H layer in adjacent pairs, P layer in adjacent pairs, then the IQFT's
    # H + CP pairs and shared-control CP pairs
    assert k.count("FusedPairTransformation") > 0
    assert len(qc.transformations) < len(W.encode_value_circuit(6, 4.7).transformations)


@pytest.mark.parametrize("build,fuse", [
    (lambda: W.encode_value_circuit(10, 4.7), FU.fuse_circuit_specialized_pairs),
    (lambda: W.encode_value_circuit(9, 300.25), FU.fuse_circuit),
    (lambda: W.random_layered_circuit(9, 4, seed=3), FU.fuse_circuit),
    (lambda: W.random_layered_circuit(8, 3, seed=4), FU.fuse_circuit_specialized_pairs),
    (lambda: W.qft_circuit(9), FU.fuse_circuit_specialized_pairs),
    (lambda: W.qft_circuit(8), FU.fuse_circuit),
])
def test_fused_circuit_gives_the_same_state_on_the_oracle(build, fuse):
    qc = build()
    fq = fuse(qc)
    re, im = W.random_normal_state(qc.num_qubits, 5)
    a = O.run(qc, re, im)
    b = O.run(fq, re, im)
    assert np.max(np.abs((a[0] - b[0]) + 1j * (a[1] - b[1]))) <= TOL


def test_contiguous_pairs_absorb_gates_on_the_pair():
    qc = bfy.QuantumCircuit(5)
    qc.h(1)
    qc.rx(2, 0.4)        # adjacent: pair (1, 2)
    qc.ry(1, 0.2)        # on the pair: absorbed
    qc.h(4)              # elsewhere: pair flushed, H(4) pending
    qc.cx(3, 4)          # controlled: flushes the pending H, passes through
    out = FU.fuse_contiguous_target_pairs(qc.transformations)
    assert kinds(out) == ["UnitaryTransformation", "GateTransformation", "GateTransformation"]
    u = out[0]
    assert u.target == 1 and u.m == 2
    expect = FU.gate_to_matrix4x4(bfy.RY(0.2), 1, 1) @ FU.gate_to_matrix4x4(bfy.RX(0.4), 1, 2) @ \
        FU.gate_to_matrix4x4(bfy.H, 1, 1)
    assert np.allclose(u.u.reshape(4, 4), expect)
    # value check through the oracle
    re, im = W.random_normal_state(5, 2)
    a, b = O.run(qc, re, im), O.run(FU.fuse_circuit(qc), re, im)
    assert np.max(np.abs(a[0] - b[0])) <= TOL and np.max(np.abs(a[1] - b[1])) <= TOL


def test_p_run_collapse_keeps_the_angle_sum_exactly():
    qc = bfy.QuantumCircuit(3)
    for a in (math.pi / 3, math.pi / 7, -0.2):
        qc.p(0, a)
    (g,) = FU.fuse_same_target_gates(qc.transformations)
    assert g.gate_info.arg == (math.pi / 3 + math.pi / 7) + -0.2


def records(qc):
    """A circuit's records as the oracle's fuse() reports them."""
    arr, cnt, keep = qc.to_ops()
    out = []
    for o in arr[:cnt]:
        d = {"kind": o.kind, "gate": o.gate, "target": o.target, "target2": o.target2, "controls": o.controls,
             "ncontrols": o.ncontrols, "flags": o.flags, "arg": o.arg, "mat": list(o.mat)}
        if o.kind in (bfy.F.BF_OP_UNITARY, bfy.F.BF_OP_CUNITARY):
            dim = 1 << o.target2
            flat = np.ctypeslib.as_array(o.data, shape=(2 * dim * dim,)).copy()
            d["data"] = flat[0::2] + 1j * flat[1::2]
        out.append(d)
    del keep
    return out


@pytest.mark.parametrize("build", [
    lambda: W.encode_value_circuit(12, 4.7),
    lambda: W.random_layered_circuit(11, 5, seed=2),
    lambda: W.qft_circuit(10),
    lambda: W.grover_circuit(6, 17),
])
@pytest.mark.parametrize("mode", [O.FUSE_CIRCUIT, O.FUSE_SPECIALIZED_PAIRS])
def test_host_rewrite_equals_the_oracle_restatement(build, mode):
    """The host mirror's rewrite and the oracle's independent restatement
    produce the same records: kinds, qubits, flags and angles exactly, the
    unitaries' matrices to the last bits of their products."""
    qc = build()
    fq = (FU.fuse_circuit if mode == O.FUSE_CIRCUIT else FU.fuse_circuit_specialized_pairs)(qc)
    mine, theirs = records(fq), O.fuse(qc, mode)
    assert len(mine) == len(theirs)
    for a, b in zip(mine, theirs):
        for key in ("kind", "target", "target2", "controls", "ncontrols", "flags"):
            assert a[key] == b[key], (key, a, b)
        if a["kind"] == bfy.F.BF_OP_GATE:
            assert a["gate"] == b["gate"] and a["arg"] == b["arg"] and a["mat"] == b["mat"]
        elif "data" in a:
            assert np.max(np.abs(a["data"] - b["data"])) <= 1e-15
