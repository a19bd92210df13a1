"""Host-side circuit fusion rewrites, restating Butterfly's
butterfly/core/transformations_fusion.mojo.

These passes rewrite a circuit's transformation list before `execute`; the
reference's fused benchmark runs `fuse_circuit_specialized_pairs` on the
value-encoding circuit and then executes the result
(benches/bench_value_encoding_strategies_qiskit.mojo:22-39).  They produce
the transformation kinds the engine accepts at its boundary:
FusedPairTransformation (a gate record flagged BF_OPF_FUSE_WITH_NEXT and its
partner), UnitaryTransformation on one or two adjacent qubits and
ControlledUnitaryTransformation on one.  The engine does its own fusion
(shared-memory tile passes and tensor-core blocks), so these rewrites matter
for drop-in parity: a circuit the reference fused must give the same state.

Conventions kept from the reference (they decide the produced matrices):
  - a 4x4 matrix on the adjacent pair (q_low, q_low + 1) indexes its basis as
    b0 + 2 b1, b0 the bit of q_low (transformations_fusion.mojo:51-95);
  - products accumulate later gates on the left: M <- G_next M (:24-33,
    :594-605, :643-650);
  - a run of P gates on one target (same control) collapses to P(sum of
    angles) (:470-477, :381-392).
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from .butterfly import (ControlKind, ControlledUnitaryTransformation, FusedPairTransformation, GateInfo, GateKind,
                        GateTransformation, QuantumCircuit, UnitaryTransformation)

_I2 = np.eye(2, dtype=np.complex128)


# ---- matrices (transformations_fusion.mojo:24-104) ---------------------------
def mul_gate(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """a . b for 2x2 gates (:24-33)."""
    return np.asarray(a, dtype=np.complex128) @ np.asarray(b, dtype=np.complex128)


def gate_to_matrix4x4(gate: np.ndarray, q_low: int, target: int) -> np.ndarray:
    """The 2x2 `gate` on `target` as a 4x4 on (q_low, q_low + 1) (:51-67):
    acting on bit b0 when target == q_low, else on bit b1."""
    g = np.asarray(gate, dtype=np.complex128)
    return np.kron(_I2, g) if target == q_low else np.kron(g, _I2)


def controlled_gate_to_matrix4x4(gate: np.ndarray, q_low: int, control: int, target: int) -> np.ndarray:
    """The 2x2 `gate` on `target` controlled by `control`, both in the pair
    (q_low, q_low + 1), as a 4x4 (:69-95)."""
    g = np.asarray(gate, dtype=np.complex128)
    m = np.zeros((4, 4), dtype=np.complex128)
    for col in range(4):
        bits = [col & 1, col >> 1]
        ctrl_bit = bits[0] if control == q_low else bits[1]
        tpos = 0 if target == q_low else 1
        if ctrl_bit == 0:
            m[col, col] = 1.0
            continue
        for out_t in range(2):
            ob = list(bits)
            ob[tpos] = out_t
            m[ob[0] + 2 * ob[1], col] = g[out_t, bits[tpos]]
    return m


def _control_of(g: GateTransformation) -> int:
    return g.controls[0] if g.kind == ControlKind.SINGLE_CONTROL else 0


def gate_bounds(g: GateTransformation) -> tuple[int, int]:
    """Lowest and highest qubit of a gate with at most one control (:106-117)."""
    qs = [g.target] + ([g.controls[0]] if g.kind == ControlKind.SINGLE_CONTROL else [])
    return min(qs), max(qs)


def _is(g: GateTransformation, kind: int, ck: int) -> bool:
    return g.kind == ck and g.gate_info.kind == kind


def is_h_gate(g) -> bool:
    return _is(g, GateKind.H, ControlKind.NO_CONTROL)


def is_p_gate(g) -> bool:
    return _is(g, GateKind.P, ControlKind.NO_CONTROL)


def is_cp_gate(g) -> bool:
    return _is(g, GateKind.P, ControlKind.SINGLE_CONTROL)


def is_special_pair_gate(g: GateTransformation) -> bool:
    """H or P without controls, or P with one control (:119-127)."""
    return is_h_gate(g) or is_p_gate(g) or is_cp_gate(g)


def pair_matrix(g: GateTransformation, q_low: int, q_high: int) -> Optional[np.ndarray]:
    """try_pair_matrix (:129-161): the 4x4 of a special-pair gate whose qubits
    all lie in {q_low, q_high}, else None."""
    if not is_special_pair_gate(g):
        return None
    pair = (q_low, q_high)
    if g.kind == ControlKind.NO_CONTROL:
        return gate_to_matrix4x4(g.gate_info.gate, q_low, g.target) if g.target in pair else None
    c = g.controls[0]
    if c == g.target or c not in pair or g.target not in pair:
        return None
    return controlled_gate_to_matrix4x4(g.gate_info.gate, q_low, c, g.target)


# ---- special pairs (transformations_fusion.mojo:181-219, 312-333) -------------
def can_fuse_special_pair(t0: GateTransformation, t1: GateTransformation) -> bool:
    """Two CPs sharing their control on different targets; or, when the two
    gates' qubits span exactly two adjacent qubits, HH, PP, H then CP, or CP
    then H (:181-219)."""
    if ControlKind.MULTI_CONTROL in (t0.kind, t1.kind):
        return False
    if is_cp_gate(t0) and is_cp_gate(t1) and t0.controls[0] == t1.controls[0] and t0.target != t1.target:
        return True
    lo0, hi0 = gate_bounds(t0)
    lo1, hi1 = gate_bounds(t1)
    if max(hi0, hi1) - min(lo0, lo1) != 1:
        return False
    return ((is_h_gate(t0) and is_h_gate(t1)) or (is_p_gate(t0) and is_p_gate(t1)) or
            (is_h_gate(t0) and is_cp_gate(t1)) or (is_cp_gate(t0) and is_h_gate(t1)))


def fuse_special_pair_gates(transformations: list) -> list:
    """Consecutive gate pairs that can_fuse_special_pair accepts become one
    FusedPairTransformation, scanning left to right without overlap
    (:312-333)."""
    out, i, n = [], 0, len(transformations)
    while i < n:
        tr = transformations[i]
        if (i + 1 < n and isinstance(tr, GateTransformation) and isinstance(transformations[i + 1], GateTransformation)
                and can_fuse_special_pair(tr, transformations[i + 1])):
            out.append(FusedPairTransformation(tr, transformations[i + 1]))
            i += 2
            continue
        out.append(tr)
        i += 1
    return out


# ---- runs on one target (transformations_fusion.mojo:335-392, 427-537) --------
class _TargetRun:
    """Consecutive gates with the same target, control kind and control,
    multiplied into one 2x2; a run of P gates keeps the sum of its angles."""

    def __init__(self, g: GateTransformation):
        self.first = g
        self.target, self.ck, self.control = g.target, g.kind, _control_of(g)
        self.product = np.array(g.gate_info.gate, dtype=np.complex128)
        self.count = 1
        self.phase = g.gate_info.kind == GateKind.P and g.gate_info.arg is not None
        self.phase_sum = g.gate_info.arg if self.phase else 0.0

    def accepts(self, g: GateTransformation) -> bool:
        return g.target == self.target and g.kind == self.ck and _control_of(g) == self.control

    def add(self, g: GateTransformation) -> None:
        self.product = mul_gate(g.gate_info.gate, self.product)
        self.count += 1
        if self.phase and g.gate_info.kind == GateKind.P and g.gate_info.arg is not None:
            self.phase_sum += g.gate_info.arg
        else:
            self.phase = False

    def emit(self, out: list) -> None:
        controls = [self.control] if self.ck == ControlKind.SINGLE_CONTROL else []
        if self.phase:
            out.append(GateTransformation(controls, self.target, GateInfo(GateKind.P, self.phase_sum)))
        elif self.count == 1:
            out.append(GateTransformation(controls, self.target, self.first.gate_info))
        elif self.ck == ControlKind.NO_CONTROL:
            out.append(UnitaryTransformation(self.product.reshape(-1), self.target, 1, "fused"))
        else:
            out.append(ControlledUnitaryTransformation(self.product.reshape(-1), self.target, self.control, 1,
                                                       "fused_ctrl"))


def fuse_same_target_gates(transformations: list) -> list:
    """Runs of gates on one target (same control kind and control) become one
    gate: P(sum) for a run of P gates, the original gate for a run of one,
    else a 1-qubit (controlled) unitary of their product.  Multi-controlled
    gates and every other transformation end a run and pass through
    (:427-537)."""
    out: list = []
    run: Optional[_TargetRun] = None
    for tr in transformations:
        if isinstance(tr, GateTransformation) and tr.kind != ControlKind.MULTI_CONTROL:
            if run is not None and run.accepts(tr):
                run.add(tr)
                continue
            if run is not None:
                run.emit(out)
            run = _TargetRun(tr)
            continue
        if run is not None:
            run.emit(out)
            run = None
        out.append(tr)
    if run is not None:
        run.emit(out)
    return out


# ---- adjacent-qubit pairs (transformations_fusion.mojo:394-425, 539-876) -------
class _PairRun:
    """A pending gate, which becomes a pair once a gate on the adjacent qubit
    (or, specialised, a special gate spanning the same two qubits) follows;
    the pair then absorbs every later gate that stays on its two qubits."""

    def __init__(self, g: GateTransformation):
        self.pending = g
        self.matrix: Optional[np.ndarray] = None
        self.low = self.high = 0

    def emit(self, out: list) -> None:
        if self.matrix is None:
            g = self.pending
            controls = [g.controls[0]] if g.kind == ControlKind.SINGLE_CONTROL else []
            out.append(GateTransformation(controls, g.target, g.gate_info))
        else:
            out.append(UnitaryTransformation(self.matrix.reshape(-1), self.low, 2, "fused_pair"))


def _fuse_pairs(transformations: list, specialized: bool) -> list:
    out: list = []
    run: Optional[_PairRun] = None

    def flush():
        nonlocal run
        if run is not None:
            run.emit(out)
            run = None

    for tr in transformations:
        passes = not isinstance(tr, GateTransformation)
        if not passes:
            if specialized:
                passes = tr.kind == ControlKind.MULTI_CONTROL or not is_special_pair_gate(tr)
            else:
                passes = tr.kind != ControlKind.NO_CONTROL
        if passes:
            flush()
            out.append(tr)
            continue
        if run is None:
            run = _PairRun(tr)
            continue
        if run.matrix is None:
            p = run.pending
            same = (tr.target == p.target and (not specialized or (tr.kind == p.kind and
                                                                   _control_of(tr) == _control_of(p))))
            if not same:
                if specialized:
                    lo = min(gate_bounds(p)[0], gate_bounds(tr)[0])
                    hi = max(gate_bounds(p)[1], gate_bounds(tr)[1])
                    if hi - lo == 1:
                        m0, m1 = pair_matrix(p, lo, hi), pair_matrix(tr, lo, hi)
                        if m0 is not None and m1 is not None:
                            run.matrix, run.low, run.high = m1 @ m0, lo, hi
                            continue
                elif abs(tr.target - p.target) == 1:
                    lo, hi = min(p.target, tr.target), max(p.target, tr.target)
                    run.matrix = gate_to_matrix4x4(tr.gate_info.gate, lo, tr.target) @ \
                        gate_to_matrix4x4(p.gate_info.gate, lo, p.target)
                    run.low, run.high = lo, hi
                    continue
            flush()
            run = _PairRun(tr)
            continue
        if specialized:
            m = pair_matrix(tr, run.low, run.high)
        else:
            m = gate_to_matrix4x4(tr.gate_info.gate, run.low, tr.target) if tr.target in (run.low, run.high) \
                else None
        if m is not None:
            run.matrix = m @ run.matrix
            continue
        flush()
        run = _PairRun(tr)
    flush()
    return out


def fuse_contiguous_target_pairs(transformations: list) -> list:
    """Uncontrolled gates on adjacent qubits become one 4x4 unitary on the
    pair, absorbing the later uncontrolled gates on its two qubits;
    controlled gates and other transformations end the pair and pass
    through (:539-687)."""
    return _fuse_pairs(transformations, specialized=False)


def fuse_contiguous_target_pairs_specialized(transformations: list) -> list:
    """The same for the special-pair gates (H, P, CP), whose qubits,
    controls included, must lie on the adjacent pair; other gates end the
    pair and pass through (:689-876)."""
    return _fuse_pairs(transformations, specialized=True)


# ---- entry points (transformations_fusion.mojo:879-908) -----------------------
def fuse_transformations(transformations: list) -> list:
    return fuse_same_target_gates(fuse_contiguous_target_pairs(transformations))


def fuse_transformations_specialized_pairs(transformations: list) -> list:
    return fuse_same_target_gates(fuse_special_pair_gates(transformations))


def _rewritten(circuit: QuantumCircuit, transformations: list) -> QuantumCircuit:
    out = QuantumCircuit(circuit.num_qubits)
    out.registers = list(circuit.registers)
    out.transformations = transformations
    return out


def fuse_circuit(circuit: QuantumCircuit) -> QuantumCircuit:
    """A copy of `circuit` with adjacent-pair and same-target fusion (:892-898)."""
    return _rewritten(circuit, fuse_transformations(list(circuit.transformations)))


def fuse_circuit_specialized_pairs(circuit: QuantumCircuit) -> QuantumCircuit:
    """A copy of `circuit` with special-pair and same-target fusion, as the
    reference's fused value-encoding benchmark runs it (:900-908)."""
    return _rewritten(circuit, fuse_transformations_specialized_pairs(list(circuit.transformations)))
