"""CPU tests of the C ABI: the library loads, exports exactly what
include/bfgpu.h declares, and its host-only logic (validation, planning)
behaves like the reference's validate_circuit.  No kernel is launched."""
import ctypes as C
import math
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import workloads as W

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    text = (ROOT / "include" / "bfgpu.h").read_text()
    return set(re.findall(r"^int (bf_\w+)\(", text, flags=re.M))


def test_library_exports_every_declared_symbol():
    lib = F.lib()
    declared = header_functions()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(F.SIGNATURES), declared ^ set(F.SIGNATURES)


def test_library_exports_nothing_undeclared():
    out = subprocess.run(["nm", "-D", "--defined-only", str(F.LIB_PATH)], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("nm unavailable")
    exported = {l.split()[-1] for l in out.stdout.splitlines() if re.search(r" T bf_", l)}
    assert exported == header_functions()


def test_struct_layouts():
    assert C.sizeof(F.bf_op) == 128
    assert C.sizeof(F.bf_exec_opts) == 32
    v = C.c_int32()
    F.check(F.lib().bf_version(C.byref(v)))
    assert v.value == 1


def test_exec_opts_defaults():
    o = F.bf_exec_opts()
    F.check(F.lib().bf_exec_opts_init(C.byref(o)))
    assert (o.strategy, o.validate, o.specialized, o.tile_qubits, o.sync) == (9, 1, 127, 0, 0)
    assert o.tensor_blocks == 1 and o.plan_dtype == 0


def test_state_create_rejects_bad_arguments_without_device():
    h = C.c_void_p()
    assert F.lib().bf_state_create(0, 0, C.byref(h)) == F.BF_EINVAL
    assert "num_qubits" in F.last_error()
    assert F.lib().bf_state_create(10, 7, C.byref(h)) == F.BF_EINVAL
    assert "dtype" in F.last_error()


# ---- validate_circuit (executors.mojo:90-185) --------------------------------
@pytest.mark.parametrize("build,msg", [
    (lambda qc: qc.h(9), "Target out of bounds: 9"),
    (lambda qc: qc.h(-1), "Target out of bounds: -1"),
    (lambda qc: qc.cx(7, 1), "Control out of bounds: 7"),
    (lambda qc: qc.unitary(np.eye(4), 3, 2), "Target range out of bounds"),
    (lambda qc: qc.c_unitary(np.eye(4), 1, 0, 2), "Control overlaps target range"),
    (lambda qc: qc.swap(0, 4), "Target out of bounds: 4"),
    (lambda qc: qc.qubit_reversal([1, 5]), "Target out of bounds: 5"),
    (lambda qc: bfy.permute_qubits(qc, [0, 1, 2]), "Permutation size mismatch: 3"),
    (lambda qc: bfy.permute_qubits(qc, [0, 1, 1, 2]), "Duplicate permutation value: 1"),
    (lambda qc: bfy.bit_reverse(qc, [1, 1]), "Duplicate target: 1"),
])
def test_validation_messages(build, msg):
    qc = bfy.QuantumCircuit(4)
    build(qc)
    with pytest.raises(F.BFError, match=msg) as e:
        bfy.validate(qc)
    assert e.value.code == F.BF_EINVAL


def test_validation_accepts_valid_circuits():
    for qc in (W.qft_circuit(8), W.random_layered_circuit(9, 3, 1), W.grover_circuit(5, 3, 1),
               W.encode_value_circuit(7, 4.7)):
        bfy.validate(qc)


def test_control_kind_mismatch_is_rejected():
    qc = bfy.QuantumCircuit(4)
    qc.cx(1, 2)
    arr, n, keep = qc.to_ops()
    arr[0].ncontrols = 2
    assert F.lib().bf_validate(4, arr, n) == F.BF_EINVAL
    assert "control kind mismatch" in F.last_error()


# ---- planner ------------------------------------------------------------------
def stats(qc, strategy=bfy.ExecutionStrategy.GPU_FUSED, K=11):
    ctx = bfy.ExecContext()
    ctx.execution_strategy = strategy
    ctx.gpu_tile_qubits = K
    return bfy.plan_stats(qc, ctx)


def test_per_gate_plan_launches_one_kernel_per_gate():
    qc = W.random_layered_circuit(12, 2, 0)
    s = stats(qc, bfy.ExecutionStrategy.GPU)
    assert s["tile_passes"] == 0 and s["gate_kernels"] == len(qc.transformations)
    # 24 dense U3 (2S each) + 12 CX (S each)
    assert math.isclose(s["bytes_in_S"], 24 * 2 + 12 * 1)


def test_qft20_fuses_to_few_passes():
    qc = W.qft_circuit(20)
    s = stats(qc, K=11)
    # 20 H spread over the qubits: 6 free tile slots beside the 5 low qubits
    assert s["tile_passes"] <= 4 and s["gate_kernels"] == 0 and s["other_passes"] == 1
    unfused = stats(qc, bfy.ExecutionStrategy.GPU)
    assert unfused["bytes_in_S"] == pytest.approx(20 * 2 + 190 * 0.5 + 2)


@pytest.mark.parametrize("K", [1, 2, 3, 4, 5, 6, 8, 10, 11, 12, 13])
def test_random_layered_pass_count_shrinks_with_width(K):
    qc = W.random_layered_circuit(30, 40, 0)
    s = stats(qc, K=K)
    total = s["tile_passes"] + s["gate_kernels"]
    assert 0 < total < 1800
    assert s["bytes_in_S"] < 3000


@pytest.mark.parametrize("n,K", [(15, 5), (15, 1), (4, 13), (5, 5), (6, 5), (3, 2)])
def test_planner_always_progresses(n, K):
    qc = W.random_layered_circuit(n, 4, 1)
    qc.transformations += W.qft_circuit(n).transformations
    s = stats(qc, K=K)
    assert s["tile_passes"] + s["gate_kernels"] > 0


def test_wider_tiles_move_fewer_bytes():
    qc = W.random_layered_circuit(30, 10, 0)
    b = [stats(qc, K=K)["bytes_in_S"] for K in (7, 9, 11, 13)]
    assert b == sorted(b, reverse=True)


@pytest.mark.parametrize("dtype,max_passes,max_blocks", [("c128", 52, 130), ("c64", 52, 132)])
def test_layered_30q_plan_quality(dtype, max_passes, max_blocks):
    """The planner's tile search on the benchmark circuit: first-come tiles
    needed 74 passes and 185 blocks; most-work tiles 48 passes and 162 blocks;
    block-rate tiles about 51 passes and 125 blocks."""
    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    s = bfy.plan_stats(W.random_layered_circuit(30, 40, 0), ctx, dtype)
    assert s["tile_passes"] <= max_passes and 0 < s["blocks"] <= max_blocks
    assert s["block_passes"] >= s["tile_passes"] - 2


def test_cuda_core_plan_takes_the_most_work_per_pass():
    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    ctx.gpu_tensor_blocks = False
    ctx.gpu_tile_qubits = 12
    s = bfy.plan_stats(W.random_layered_circuit(30, 40, 0), ctx)
    assert s["tile_passes"] <= 50 and s["block_passes"] == 0


def test_diagonal_gates_never_constrain_tiles():
    qc = bfy.QuantumCircuit(24)
    for q in range(24):
        qc.h(q % 5)
        qc.cp(23 - q, q, 0.1 * q)
        qc.p(q, 0.2)
    s = stats(qc, K=6)
    assert s["tile_passes"] == 1 and s["gate_kernels"] == 0


def test_batch_workload_shape():
    circs = W.batch_workload(count=64, seed=1)
    ns = [c.num_qubits for c in circs]
    assert min(ns) >= 8 and max(ns) <= 20 and len(circs) == 64
    # gate transformations only (a batch takes nothing else)
    for c in circs:
        assert all(isinstance(t, bfy.GateTransformation) for t in c.transformations)


def test_random_op_records_are_validated_without_crashing():
    """Random op records (pointers null, counts and fields random): the
    validator and the host planner return a status, never crash."""
    rng = np.random.Generator(np.random.PCG64(31))
    statuses = set()
    for trial in range(2000):
        nops = int(rng.integers(1, 6))
        arr = (F.bf_op * nops)()
        for o in arr:
            o.kind = int(rng.integers(-2, 16))
            o.gate = int(rng.integers(-2, 12))
            o.target = int(rng.integers(-3, 70))
            o.target2 = int(rng.integers(-3, 10))
            o.controls = int(rng.integers(0, 2 ** 63))
            o.ncontrols = int(rng.integers(-1, 5))
            o.flags = int(rng.integers(0, 4))
            o.arg = float(rng.normal())
            o.nqubits = int(rng.integers(-2, 5))
            for k in range(8):
                o.mat[k] = float(rng.normal())
        n = int(rng.integers(-1, 42))
        statuses.add(F.lib().bf_validate(n, arr, nops))
        ctx = F.bf_exec_opts()
        F.lib().bf_exec_opts_init(C.byref(ctx))
        t, g, x, bp, nb = (C.c_int64() for _ in range(5))
        b = C.c_double()
        statuses.add(F.lib().bf_plan_stats(n, arr, nops, C.byref(ctx), C.byref(t), C.byref(g), C.byref(x),
                                           C.byref(b), C.byref(bp), C.byref(nb)))
    assert F.BF_EINVAL in statuses


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_fuse_circuit_layered_30q_plans_unitaries_into_block_passes(dtype):
    """The reference's fuse_circuit turns the benchmark circuit's neighbour
    pairs into 4x4 unitaries; they stay inside the fused run (no pass of their
    own) and nearly every pass runs as tensor-core blocks."""
    from code_mojo_gb300 import fusion as FU
    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    s = bfy.plan_stats(FU.fuse_circuit(W.random_layered_circuit(30, 40, 0)), ctx, dtype)
    assert s["other_passes"] == 0 and s["gate_kernels"] == 0
    assert s["block_passes"] >= s["tile_passes"] - 2 and s["tile_passes"] <= 110
