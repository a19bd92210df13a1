"""Python mirror of Butterfly's circuit / execute API, backed by libbfgpu.

Names, argument meaning and error behaviour follow the reference:
  * gates and GateInfo ........ butterfly/core/gates.mojo:5-195
  * Circuit builder ........... butterfly/core/circuit.mojo:259-961
  * classical transforms ...... butterfly/core/quantum_circuit.mojo:99-136
  * ExecContext / strategies .. butterfly/utils/context.mojo:12-116
  * execute ................... butterfly/core/executors.mojo:723-730
so that the tests read like the reference's own.  The state lives on the GPU
(QuantumState wraps a bf_state); execute() flattens the circuit into bf_op
records and calls bf_execute.  There is no CPU execution path here.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _ffi as F

# ---------------------------------------------------------------------------
# kinds and strategies


class GateKind:
    H, P, X, Y, Z, RX, RY, RZ, CUSTOM = range(9)
    names = ["H", "P", "X", "Y", "Z", "RX", "RY", "RZ", "CUSTOM"]


class ControlKind:
    NO_CONTROL, SINGLE_CONTROL, MULTI_CONTROL = 0, 1, 2


class ExecutionStrategy:
    SCALAR = 0
    SCALAR_PARALLEL = 1
    SIMD = 2
    SIMD_PARALLEL = 3
    GRID = 4
    GRID_PARALLEL = 5
    GRID_FUSED = 6
    GRID_PARALLEL_FUSED = 7
    GPU = 8          # one kernel per transformation
    GPU_FUSED = 9    # shared-memory tile passes


class ExecContext:
    """Runtime options (context.mojo:67-116) plus the GPU strategy knobs."""

    def __init__(self) -> None:
        self.threads = 0
        self.quantum_simd_parallel_chunks = 0
        self.simd_use_specialized_h = True
        self.simd_use_specialized_p = True
        self.simd_use_specialized_cp = True
        self.simd_use_specialized_x = True
        self.simd_use_specialized_cx = True
        self.simd_use_specialized_ry = True
        self.simd_use_specialized_cry = True
        self.grid_col_bits_min = 3
        self.grid_col_bits_slack = 3
        self.validate_circuit = True
        self.execution_strategy = ExecutionStrategy.GPU_FUSED
        self.gpu_tile_qubits = 0     # fusion width of a tile pass (0 = default)
        self.gpu_tensor_blocks = True   # 5-qubit blocks on the tensor cores where cheaper (3xTF32 / bf16 digits)
        self.gpu_renormalize = True  # complex64: restore the input norm after the circuit
        self.gpu_sync = True         # block until the device has finished

    def copy(self) -> "ExecContext":
        c = ExecContext()
        c.__dict__.update(self.__dict__)
        return c

    def specialized_mask(self) -> int:
        flags = [self.simd_use_specialized_h, self.simd_use_specialized_p, self.simd_use_specialized_cp,
                 self.simd_use_specialized_x, self.simd_use_specialized_cx, self.simd_use_specialized_ry,
                 self.simd_use_specialized_cry]
        return sum(1 << i for i, f in enumerate(flags) if f)


# ---------------------------------------------------------------------------
# gate matrices (gates.mojo:5-61); cis (utils/common.mojo:8-9)

sq_half_re = math.sqrt(0.5)


def cis(theta: float) -> complex:
    return complex(math.cos(theta), math.sin(theta))


def _g(a, b, c, d) -> np.ndarray:
    return np.array([[a, b], [c, d]], dtype=np.complex128)


H = _g(sq_half_re, sq_half_re, sq_half_re, -sq_half_re)
X = _g(0, 1, 1, 0)
Y = _g(0, -1j, 1j, 0)
Z = _g(1, 0, 0, -1)


def P(theta: float) -> np.ndarray:
    return _g(1, 0, 0, cis(theta))


def RX(theta: float) -> np.ndarray:
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return _g(c, complex(0, -s), complex(0, -s), c)


def RY(theta: float) -> np.ndarray:
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return _g(c, -s, s, c)


def RZ(theta: float) -> np.ndarray:
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return _g(complex(c, -s), 0, 0, complex(c, s))


def U3(theta: float, phi: float, lam: float) -> np.ndarray:
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return _g(complex(c, 0), -cis(lam) * s, cis(phi) * s, cis(phi + lam) * c)


def U2(phi: float, lam: float) -> np.ndarray:
    return U3(math.pi / 2, phi, lam)


def U1(lam: float) -> np.ndarray:
    return U3(0, 0, lam)


_KIND_MATRIX = {GateKind.H: lambda a: H, GateKind.P: P, GateKind.X: lambda a: X, GateKind.Y: lambda a: Y,
                GateKind.Z: lambda a: Z, GateKind.RX: RX, GateKind.RY: RY, GateKind.RZ: RZ}


class GateInfo:
    """GateInfo (gates.mojo:137-175).  CUSTOM requires an explicit matrix (the
    reference silently substitutes H when it is missing, gates.mojo:125-135)."""

    def __init__(self, kind: int, arg: Optional[float] = None, gate: Optional[np.ndarray] = None,
                 name: Optional[str] = None):
        self.kind = kind
        self.name = name or GateKind.names[kind]
        if kind == GateKind.CUSTOM:
            if gate is None:
                raise ValueError("CUSTOM gate requires a 2x2 matrix")
            self.gate = np.asarray(gate, dtype=np.complex128).reshape(2, 2)
            self.arg = None
        else:
            fn = _KIND_MATRIX[kind]
            if kind in (GateKind.P, GateKind.RX, GateKind.RY, GateKind.RZ):
                if arg is None:
                    raise ValueError(f"{self.name} needs an angle")
                self.arg = float(arg)
                self.gate = fn(self.arg)
            else:
                self.arg = None
                self.gate = fn(None)

    def __repr__(self) -> str:
        return f"{self.name}({self.arg})" if self.arg is not None else self.name


H_Gate = GateInfo(GateKind.H)
X_Gate = GateInfo(GateKind.X)
Y_Gate = GateInfo(GateKind.Y)
Z_Gate = GateInfo(GateKind.Z)


def P_Gate(theta: float) -> GateInfo:
    return GateInfo(GateKind.P, theta)


def RX_Gate(theta: float) -> GateInfo:
    return GateInfo(GateKind.RX, theta)


def RY_Gate(theta: float) -> GateInfo:
    return GateInfo(GateKind.RY, theta)


def RZ_Gate(theta: float) -> GateInfo:
    return GateInfo(GateKind.RZ, theta)


def Custom_Gate(gate: np.ndarray, name: str = "CUSTOM") -> GateInfo:
    return GateInfo(GateKind.CUSTOM, gate=gate, name=name)


# ---------------------------------------------------------------------------
# transformations (circuit.mojo:46-239)


class GateTransformation:
    def __init__(self, controls: Sequence[int], target: int, gate_info: GateInfo):
        self.controls = list(controls)
        self.target = target
        self.gate_info = gate_info
        n = len(self.controls)
        self.kind = ControlKind.NO_CONTROL if n == 0 else (
            ControlKind.SINGLE_CONTROL if n == 1 else ControlKind.MULTI_CONTROL)


class FusedPairTransformation:
    def __init__(self, first: GateTransformation, second: GateTransformation):
        self.first = first
        self.second = second


class SwapTransformation:
    def __init__(self, a: int, b: int):
        self.a, self.b = a, b


class QubitReversalTransformation:
    def __init__(self, targets: Sequence[int] = ()):
        self.targets = list(targets)


class UnitaryTransformation:
    def __init__(self, u, target: int, m: int, name: str = "unitary"):
        self.u = np.asarray(u, dtype=np.complex128).reshape(-1)
        self.target, self.m, self.name = target, m, name


class ControlledUnitaryTransformation:
    def __init__(self, u, target: int, control: int, m: int, name: str = "unitary"):
        self.u = np.asarray(u, dtype=np.complex128).reshape(-1)
        self.target, self.control, self.m, self.name = target, control, m, name


class ClassicalTransformation:
    """The classical transforms on the hot path: BITREV, PERMUTE and SWAP
    (quantum_circuit.mojo:99-123), the Grover diffuser / inversion about
    |0> (grover_classical.mojo:262-326) and Shor's modular exponentiation
    MOD_EXP / MOD_EXP_INV with targets [n_exp, n_value, a, N]
    (algos/shor.mojo:56-166)."""

    def __init__(self, name: str, targets: Sequence[int]):
        if name not in ("BITREV", "PERMUTE", "SWAP", "GROVER_DIFFUSER", "GROVER_INVERSION_0", "MOD_EXP",
                        "MOD_EXP_INV"):
            raise ValueError(f"unsupported classical transform {name}")
        self.name = name
        self.targets = list(targets)


class MeasurementTransformation:
    """MeasurementTransformation (circuit.mojo:200-227): apply_measure on
    `targets`; values[k] None = free, True/False = post-selected."""

    def __init__(self, targets: Sequence[int], values=None, seed: Optional[int] = None):
        self.targets = list(targets)
        self.values = list(values) if values else [None] * len(self.targets)
        if len(self.values) != len(self.targets):
            raise ValueError("Measurement values length mismatch")
        self.seed = seed


class Register:
    def __init__(self, name: str, length: int, start: int = 0):
        self.name, self.length, self.start = name, length, start

    def __getitem__(self, i: int) -> int:
        return self.start + i


def _matrix_check(u, m: int) -> np.ndarray:
    u = np.asarray(u, dtype=np.complex128).reshape(-1)
    dim = 1 << m
    if u.size != dim * dim:
        raise ValueError(f"Unitary size mismatch. Expected {dim * dim}, got {u.size}")
    return u


class QuantumCircuit:
    """Circuit[QuantumState] (circuit.mojo:259-961)."""

    def __init__(self, num_qubits):
        if isinstance(num_qubits, Register):
            self.registers = [num_qubits]
            num_qubits = num_qubits.length
        else:
            self.registers = [Register("q", num_qubits)]
        self.num_qubits = int(num_qubits)
        self.transformations: list = []

    # -- gates ----------------------------------------------------------------
    def add(self, controls, target, gate_info: Optional[GateInfo] = None):
        """add(target, gate_info) or add(controls, target, gate_info)."""
        if gate_info is None:
            controls, target, gate_info = [], controls, target
        elif isinstance(controls, int):
            controls = [controls]
        self.transformations.append(GateTransformation(controls, target, gate_info))

    def h(self, t): self.add(t, H_Gate)
    def x(self, t): self.add(t, X_Gate)
    def y(self, t): self.add(t, Y_Gate)
    def z(self, t): self.add(t, Z_Gate)
    def p(self, t, theta): self.add(t, P_Gate(theta))
    def rx(self, t, theta): self.add(t, RX_Gate(theta))
    def ry(self, t, theta): self.add(t, RY_Gate(theta))
    def rz(self, t, theta): self.add(t, RZ_Gate(theta))
    def cp(self, c, t, theta): self.add(c, t, P_Gate(theta))
    def cx(self, c, t): self.add(c, t, X_Gate)
    def cy(self, c, t): self.add(c, t, Y_Gate)
    def cz(self, c, t): self.add(c, t, Z_Gate)
    def crx(self, c, t, theta): self.add(c, t, RX_Gate(theta))
    def cry(self, c, t, theta): self.add(c, t, RY_Gate(theta))
    def crz(self, c, t, theta): self.add(c, t, RZ_Gate(theta))
    def ccx(self, c1, c2, t): self.add([c1, c2], t, X_Gate)
    def mcp(self, controls, t, theta): self.add(list(controls), t, P_Gate(theta))

    def u3(self, t, theta, phi, lam):
        """U3 enters as a CUSTOM gate with the U3 matrix (gates.mojo:42-54)."""
        self.add(t, Custom_Gate(U3(theta, phi, lam), "U3"))

    def custom(self, t, gate, controls: Sequence[int] = ()):
        self.add(list(controls), t, Custom_Gate(gate))

    # -- other transformations -----------------------------------------------
    def swap(self, a, b): self.transformations.append(SwapTransformation(a, b))

    def qubit_reversal(self, targets: Optional[Iterable[int]] = None):
        if isinstance(targets, Register):
            targets = [targets.start + i for i in range(targets.length)]
        self.transformations.append(QubitReversalTransformation(list(targets or [])))

    def unitary(self, u, target: int, m: int = 1, name: str = "unitary"):
        self.transformations.append(UnitaryTransformation(_matrix_check(u, m), target, m, name))

    def c_unitary(self, u, control: int, target: int, m: int = 1, name: str = "unitary"):
        self.transformations.append(ControlledUnitaryTransformation(_matrix_check(u, m), target, control, m, name))

    def append_fused_pair(self, first: GateTransformation, second: GateTransformation):
        self.transformations.append(FusedPairTransformation(first, second))

    def inverse(self) -> "QuantumCircuit":
        """Circuit.inverse (circuit.mojo:945-1037): reversed order; P/RX/RY/RZ
        angles negated; H/X/Y/Z, swaps, reversals and classical permutations
        kept.  CUSTOM gates raise, as in the reference; unitaries take the
        conjugate transpose (the reference only conjugates, circuit.mojo:
        1077-1088)."""
        out = QuantumCircuit(self.num_qubits)
        out.registers = list(self.registers)
        for tr in reversed(self.transformations):
            out.transformations.append(_invert(tr))
        return out

    # -- flattening ------------------------------------------------------------
    def to_ops(self):
        """Returns (ctypes bf_op array, count, keepalive list)."""
        keep: list = []
        ops: list[F.bf_op] = []
        for tr in self.transformations:
            if isinstance(tr, FusedPairTransformation):
                a = _gate_op(tr.first)
                a.flags |= F.BF_OPF_FUSE_WITH_NEXT
                ops += [a, _gate_op(tr.second)]
            elif isinstance(tr, GateTransformation):
                ops.append(_gate_op(tr))
            elif isinstance(tr, SwapTransformation):
                ops.append(_op(F.BF_OP_SWAP, target=tr.a, target2=tr.b))
            elif isinstance(tr, QubitReversalTransformation):
                ops.append(_list_op(F.BF_OP_QREV, tr.targets, keep))
            elif isinstance(tr, UnitaryTransformation):
                ops.append(_unitary_op(F.BF_OP_UNITARY, tr.u, tr.target, tr.m, None, keep))
            elif isinstance(tr, ControlledUnitaryTransformation):
                ops.append(_unitary_op(F.BF_OP_CUNITARY, tr.u, tr.target, tr.m, tr.control, keep))
            elif isinstance(tr, MeasurementTransformation):
                vals = np.array([-1.0 if v is None else float(bool(v)) for v in tr.values], dtype=np.float64)
                keep.append(vals)
                o = _list_op(F.BF_OP_MEASURE, tr.targets, keep)
                o.data = vals.ctypes.data_as(C.POINTER(C.c_double))
                o.arg = float(-1 if tr.seed is None else tr.seed)
                ops.append(o)
            elif isinstance(tr, ClassicalTransformation):
                if tr.name == "BITREV":
                    ops.append(_list_op(F.BF_OP_BITREV, tr.targets, keep))
                elif tr.name == "PERMUTE":
                    ops.append(_list_op(F.BF_OP_PERMUTE, tr.targets, keep))
                elif tr.name == "GROVER_DIFFUSER":
                    ops.append(_list_op(F.BF_OP_GROVER_DIFFUSER, tr.targets, keep))
                elif tr.name == "GROVER_INVERSION_0":
                    ops.append(_list_op(F.BF_OP_GROVER_INVERSION0, tr.targets, keep))
                elif tr.name in ("MOD_EXP", "MOD_EXP_INV"):
                    vals = np.array([float(v) for v in tr.targets], dtype=np.float64)
                    keep.append(vals)
                    o = _op(F.BF_OP_MODEXP if tr.name == "MOD_EXP" else F.BF_OP_MODEXP_INV)
                    o.data = vals.ctypes.data_as(C.POINTER(C.c_double))
                    o.nqubits = len(vals)
                    ops.append(o)
                else:
                    if len(tr.targets) != 2:
                        raise ValueError("SWAP expects 2 targets")
                    ops.append(_op(F.BF_OP_CSWAP, target=tr.targets[0], target2=tr.targets[1]))
            else:
                raise ValueError("Unknown transformation type")
        arr = (F.bf_op * max(1, len(ops)))(*ops)
        return arr, len(ops), keep


def _op(kind, **kw) -> F.bf_op:
    o = F.bf_op()
    o.kind = kind
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _gate_op(gt: GateTransformation) -> F.bf_op:
    o = _op(F.BF_OP_GATE, gate=gt.gate_info.kind, target=gt.target)
    mask = 0
    for c in gt.controls:
        if c < 0 or c >= 64:
            raise ValueError(f"Control out of bounds: {c}")
        mask |= 1 << c
    o.controls = mask
    # ControlKind follows the list length; duplicated controls collapse in the mask
    o.ncontrols = bin(mask).count("1") if len(set(gt.controls)) == len(gt.controls) else len(gt.controls)
    o.arg = gt.gate_info.arg if gt.gate_info.arg is not None else 0.0
    g = gt.gate_info.gate
    for i, v in enumerate((g[0, 0], g[0, 1], g[1, 0], g[1, 1])):
        o.mat[2 * i] = v.real
        o.mat[2 * i + 1] = v.imag
    return o


def _list_op(kind, targets, keep) -> F.bf_op:
    arr = (C.c_int32 * max(1, len(targets)))(*targets)
    keep.append(arr)
    return _op(kind, qubits=C.cast(arr, C.POINTER(C.c_int32)), nqubits=len(targets))


def _unitary_op(kind, u, target, m, control, keep) -> F.bf_op:
    buf = np.ascontiguousarray(np.stack([u.real, u.imag], axis=-1).reshape(-1), dtype=np.float64)
    keep.append(buf)
    o = _op(kind, target=target, target2=m, data=buf.ctypes.data_as(C.POINTER(C.c_double)))
    if control is not None:
        o.controls = 1 << control
        o.ncontrols = 1
    return o


def _invert_gate(gt: GateTransformation) -> GateTransformation:
    gi = gt.gate_info
    if gi.kind in (GateKind.H, GateKind.X, GateKind.Y, GateKind.Z):
        return GateTransformation(gt.controls, gt.target, gi)
    if gi.kind in (GateKind.P, GateKind.RX, GateKind.RY, GateKind.RZ):
        return GateTransformation(gt.controls, gt.target, GateInfo(gi.kind, -gi.arg))
    raise ValueError("Custom gate inversion not implemented. Use unitary matrices for complex gates.")


def _invert(tr):
    if isinstance(tr, MeasurementTransformation):
        raise ValueError("Cannot invert circuit containing measurements")
    if isinstance(tr, GateTransformation):
        return _invert_gate(tr)
    if isinstance(tr, FusedPairTransformation):
        return FusedPairTransformation(_invert_gate(tr.second), _invert_gate(tr.first))
    if isinstance(tr, UnitaryTransformation):
        d = 1 << tr.m
        return UnitaryTransformation(tr.u.reshape(d, d).conj().T.reshape(-1), tr.target, tr.m, tr.name + "_inv")
    if isinstance(tr, ControlledUnitaryTransformation):
        d = 1 << tr.m
        return ControlledUnitaryTransformation(tr.u.reshape(d, d).conj().T.reshape(-1), tr.target, tr.control,
                                               tr.m, tr.name + "_inv")
    if isinstance(tr, ClassicalTransformation) and tr.name == "PERMUTE" and tr.targets:
        inv = [0] * len(tr.targets)
        for i, v in enumerate(tr.targets):
            inv[v] = i
        return ClassicalTransformation("PERMUTE", inv)
    if isinstance(tr, ClassicalTransformation) and tr.name in ("MOD_EXP", "MOD_EXP_INV"):
        # add_classical registers apply_modexp_inverse as MOD_EXP's inverse (algos/shor.mojo:161-166)
        return ClassicalTransformation("MOD_EXP_INV" if tr.name == "MOD_EXP" else "MOD_EXP", tr.targets)
    return tr  # swaps, reversals, bit reversal: self-inverse


# classical transforms (quantum_circuit.mojo:99-136)
def bit_reverse(circuit: QuantumCircuit, targets: Optional[Sequence[int]] = None) -> None:
    circuit.transformations.append(ClassicalTransformation("BITREV", list(targets or [])))


def permute_qubits(circuit: QuantumCircuit, order: Sequence[int]) -> None:
    circuit.transformations.append(ClassicalTransformation("PERMUTE", list(order)))


def measure(circuit: QuantumCircuit, targets: Sequence[int], values=None, seed: Optional[int] = None) -> None:
    """quantum_circuit.mojo:139-182."""
    circuit.transformations.append(MeasurementTransformation(targets, values, seed))


def grover_diffuser(circuit: QuantumCircuit, targets: Optional[Sequence[int]] = None) -> None:
    """Classical inversion about the mean over `targets` (all when empty),
    apply_grover_diffuser (grover_classical.mojo:284-326), computed as
    2*mean - x for both real and imaginary parts."""
    circuit.transformations.append(ClassicalTransformation("GROVER_DIFFUSER", list(targets or [])))


def grover_inversion_0(circuit: QuantumCircuit, targets: Optional[Sequence[int]] = None) -> None:
    """Classical phase flip of |0...0> on `targets` (grover_classical.mojo:262-281)."""
    circuit.transformations.append(ClassicalTransformation("GROVER_INVERSION_0", list(targets or [])))


def swap_tr(a: int, b: int) -> ClassicalTransformation:
    return ClassicalTransformation("SWAP", [a, b])


def mod_exp(circuit: QuantumCircuit, n_exp: int, n_value: int, a: int, modulus: int) -> None:
    """The MOD_EXP classical transform of modexp_circuit (algos/shor.mojo:156-166)."""
    circuit.transformations.append(ClassicalTransformation("MOD_EXP", [n_exp, n_value, a, modulus]))


# ---------------------------------------------------------------------------
# wire formats
def parse_qasm3_string(qasm: str) -> QuantumCircuit:
    """parse_qasm3_string (butterfly/utils/qasm3_import.mojo:52-123), parsed
    by the library (bf_qasm3_parse): a qubit declaration, then h, x, p(angle)
    and cp(angle) lines."""
    h = C.c_void_p()
    F.check(F.lib().bf_qasm3_parse(qasm.encode(), C.byref(h)))
    try:
        ops, cnt, n = C.POINTER(F.bf_op)(), C.c_int64(), C.c_int32()
        F.check(F.lib().bf_oplist_view(h, C.byref(ops), C.byref(cnt), C.byref(n)))
        qc = QuantumCircuit(n.value)
        for i in range(cnt.value):
            o = ops[i]
            gate = {F.BF_GATE_H: H_Gate, F.BF_GATE_X: X_Gate}.get(o.gate) or P_Gate(o.arg)
            if o.ncontrols:
                qc.add(int(o.controls).bit_length() - 1, o.target, gate)
            else:
                qc.add(o.target, gate)
        return qc
    finally:
        F.lib().bf_oplist_destroy(h)


def serialize(circuit) -> bytes:
    """The binary op list of a circuit (bf_ops_serialize)."""
    arr, n, keep = circuit.to_ops()
    size = C.c_size_t()
    F.check(F.lib().bf_ops_serialize(circuit.num_qubits, arr, n, None, 0, C.byref(size)))
    buf = C.create_string_buffer(max(1, size.value))
    F.check(F.lib().bf_ops_serialize(circuit.num_qubits, arr, n, buf, size.value, C.byref(size)))
    del keep
    return buf.raw[:size.value]


class OpList:
    """An op list owned by the library (bf_ops_deserialize / bf_qasm3_parse);
    executable like a circuit."""

    def __init__(self, blob: bytes):
        self._h = C.c_void_p()
        F.check(F.lib().bf_ops_deserialize(blob, len(blob), C.byref(self._h)))
        ops, cnt, n = C.POINTER(F.bf_op)(), C.c_int64(), C.c_int32()
        F.check(F.lib().bf_oplist_view(self._h, C.byref(ops), C.byref(cnt), C.byref(n)))
        self._ops, self._count, self.num_qubits = ops, cnt.value, n.value

    def __len__(self) -> int:
        return self._count

    def to_ops(self):
        return self._ops, self._count, [self]

    def close(self) -> None:
        if getattr(self, "_h", None):
            F.lib().bf_oplist_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def deserialize(blob: bytes) -> OpList:
    return OpList(blob)


# ---------------------------------------------------------------------------
# device state and execute


class QuantumState:
    """State / QuantumState (state.mojo:19-98) resident on the GPU.

    QuantumState(n) is |0...0>; dtype "c128" (FP64 storage) or "c64"."""

    def __init__(self, n: int, dtype: str = "c128"):
        self._h = C.c_void_p()
        self.dtype = dtype
        code = {"c128": F.BF_C128, "c64": F.BF_C64}[dtype]
        F.check(F.lib().bf_state_create(int(n), code, C.byref(self._h)))
        self.num_qubits = int(n)

    @classmethod
    def from_soa(cls, re: np.ndarray, im: np.ndarray, dtype: str = "c128") -> "QuantumState":
        n = int(len(re)).bit_length() - 1
        if len(re) != 1 << n or len(im) != len(re):
            raise ValueError("State size must be a power of two")
        st = cls(n, dtype)
        st.upload(re, im)
        return st

    @classmethod
    def from_complex(cls, amps: np.ndarray, dtype: str = "c128") -> "QuantumState":
        a = np.asarray(amps, dtype=np.complex128)
        return cls.from_soa(np.ascontiguousarray(a.real), np.ascontiguousarray(a.imag), dtype)

    def size(self) -> int:
        return 1 << self.num_qubits

    __len__ = size

    @property
    def handle(self) -> C.c_void_p:
        if not self._h:
            raise ValueError("state is closed")
        return self._h

    def upload(self, re: np.ndarray, im: np.ndarray) -> None:
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = np.ascontiguousarray(im, dtype=np.float64)
        if re.size != self.size() or im.size != self.size():
            raise ValueError("size mismatch")
        F.check(F.lib().bf_state_upload_soa(self.handle, re.ctypes.data, im.ctypes.data))
        F.check(F.lib().bf_state_sync(self.handle))

    def download(self) -> tuple[np.ndarray, np.ndarray]:
        re = np.empty(self.size(), dtype=np.float64)
        im = np.empty(self.size(), dtype=np.float64)
        F.check(F.lib().bf_state_download_soa(self.handle, re.ctypes.data, im.ctypes.data))
        return re, im

    def to_complex(self) -> np.ndarray:
        re, im = self.download()
        return re + 1j * im

    def set_basis(self, idx: int) -> None:
        F.check(F.lib().bf_state_set_basis(self.handle, int(idx)))

    def norm2(self) -> float:
        out = C.c_double()
        F.check(F.lib().bf_norm2(self.handle, C.byref(out)))
        return out.value

    def sync(self) -> None:
        F.check(F.lib().bf_state_sync(self.handle))

    @staticmethod
    def _values(values, n):
        if values is None:
            return None
        arr = (C.c_int8 * max(1, n))(*[(-1 if v is None else int(bool(v))) for v in values])
        return arr

    def probabilities(self, qubits: Sequence[int], values=None) -> np.ndarray:
        """Outcome probabilities of the free qubits among `qubits` (bit j of
        the outcome index = j-th free qubit); values fix the others."""
        q = (C.c_int32 * max(1, len(qubits)))(*qubits)
        v = self._values(values, len(qubits))
        nfree = len(qubits) if values is None else sum(1 for x in values if x is None)
        out = np.empty(1 << nfree, dtype=np.float64)
        F.check(F.lib().bf_probabilities(self.handle, q, v, len(qubits), out.ctypes.data))
        return out

    def measure(self, targets: Sequence[int], values=None, seed: Optional[int] = None) -> tuple[int, float]:
        """apply_measure (state.mojo:447-553): returns (outcome, probability)
        and collapses the state."""
        q = (C.c_int32 * max(1, len(targets)))(*targets)
        v = self._values(values, len(targets))
        oc, pr = C.c_uint64(), C.c_double()
        F.check(F.lib().bf_measure(self.handle, q, v, len(targets), -1 if seed is None else int(seed), C.byref(oc),
                                   C.byref(pr)))
        return oc.value, pr.value

    def inner(self, other: "QuantumState") -> complex:
        """<self|other> on the device (double-float accumulation)."""
        re, im = C.c_double(), C.c_double()
        F.check(F.lib().bf_inner(self.handle, other.handle, C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    def topk(self, k: int = 16) -> tuple[np.ndarray, np.ndarray]:
        idx = np.empty(k, dtype=np.uint64)
        pr = np.empty(k, dtype=np.float64)
        F.check(F.lib().bf_probs_topk(self.handle, k, idx.ctypes.data, pr.ctypes.data))
        return idx, pr

    def stream_ptr(self) -> int:
        p = C.c_void_p()
        F.check(F.lib().bf_state_stream(self.handle, C.byref(p)))
        return p.value or 0

    def launch_count(self, reset: bool = False) -> int:
        v = C.c_uint64()
        F.check(F.lib().bf_state_launch_count(self.handle, C.byref(v), 1 if reset else 0))
        return v.value

    PASS_CLASSES = ("gate", "tile", "block_tf32", "block_digits", "other")

    def pass_timing(self, enable: bool) -> None:
        """Bracket every pass of later executes with CUDA events on the
        state's stream (read with pass_times)."""
        F.check(F.lib().bf_state_pass_timing(self.handle, 1 if enable else 0))

    def pass_times(self) -> dict:
        """{class: (passes, summed device ms)} of the passes timed since the
        last call; waits for the state's stream."""
        n = len(self.PASS_CLASSES)
        cnt = np.zeros(n, dtype=np.int64)
        ms = np.zeros(n, dtype=np.float64)
        F.check(F.lib().bf_state_pass_times(self.handle, cnt.ctypes.data, ms.ctypes.data))
        return {k: (int(cnt[i]), float(ms[i])) for i, k in enumerate(self.PASS_CLASSES) if cnt[i]}

    def digit_tiles(self, reset: bool = False) -> tuple[int, int]:
        """(five-digit, six-digit) tiles of the complex128 digit passes run on
        this state; waits for the state's stream."""
        five, six = C.c_uint64(), C.c_uint64()
        F.check(F.lib().bf_state_digit_tiles(self.handle, C.byref(five), C.byref(six), 1 if reset else 0))
        return five.value, six.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            F.lib().bf_state_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def exec_opts(ctx: ExecContext) -> F.bf_exec_opts:
    o = F.bf_exec_opts()
    F.check(F.lib().bf_exec_opts_init(C.byref(o)))
    o.strategy = ctx.execution_strategy
    o.validate = 1 if ctx.validate_circuit else 0
    o.specialized = ctx.specialized_mask()
    o.tile_qubits = ctx.gpu_tile_qubits
    o.sync = 1 if ctx.gpu_sync else 0
    o.tensor_blocks = 1 if ctx.gpu_tensor_blocks else 0
    o.renormalize = 0 if ctx.gpu_renormalize else -1
    return o


def execute(state: QuantumState, circuit: QuantumCircuit, ctx: Optional[ExecContext] = None) -> None:
    """execute(state, circuit, ctx) (executors.mojo:723-730): runs the circuit
    on the device state in place.  Raises like the reference's validation."""
    ctx = ctx or ExecContext()
    if ctx.validate_circuit and circuit.num_qubits != state.num_qubits:
        raise F.BFError(F.BF_EINVAL, f"Circuit qubits mismatch: circuit has {circuit.num_qubits}, "
                                     f"state has {state.num_qubits}")
    arr, n, keep = circuit.to_ops()
    opts = exec_opts(ctx)
    F.check(F.lib().bf_execute(state.handle, arr, n, C.byref(opts)))
    del keep


def plan_stats(circuit: QuantumCircuit, ctx: Optional[ExecContext] = None, dtype: str = "c128") -> dict:
    """Host-only plan of a circuit for a state of `dtype`: launches and
    algorithmic bytes (units of S)."""
    ctx = ctx or ExecContext()
    arr, n, keep = circuit.to_ops()
    opts = exec_opts(ctx)
    opts.plan_dtype = F.BF_C64 if dtype == "c64" else F.BF_C128
    t, g, x, bp, nb = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    b = C.c_double()
    F.check(F.lib().bf_plan_stats(circuit.num_qubits, arr, n, C.byref(opts), C.byref(t), C.byref(g), C.byref(x),
                                  C.byref(b), C.byref(bp), C.byref(nb)))
    del keep
    return {"tile_passes": t.value, "gate_kernels": g.value, "other_passes": x.value, "bytes_in_S": b.value,
            "block_passes": bp.value, "blocks": nb.value}


def validate(circuit: QuantumCircuit, num_qubits: Optional[int] = None) -> None:
    arr, n, keep = circuit.to_ops()
    F.check(F.lib().bf_validate(num_qubits if num_qubits is not None else circuit.num_qubits, arr, n))
    del keep
