"""Circuits rewritten by the reference's fusion passes (restated in
code_mojo_gb300/fusion.py) run through the engine: the state equals the
oracle's run of the unfused circuit (complex128 within max|d amp| <= 1e-12,
complex64 within infidelity <= 1e-6).  The value-encoding circuit through
fuse_circuit_specialized_pairs is what the reference's fused benchmark
executes (benches/bench_value_encoding_strategies_qiskit.mojo:22-39)."""
import numpy as np
import pytest

from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import fusion as FU
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def run_gpu(qc, strategy, dtype="c128", state=None):
    st = bfy.QuantumState.from_soa(*state, dtype) if state is not None else bfy.QuantumState(qc.num_qubits, dtype)
    ctx = bfy.ExecContext()
    ctx.execution_strategy = strategy
    bfy.execute(st, qc, ctx)
    z = st.to_complex()
    st.close()
    return z


def oracle_of(qc, state=None):
    re, im = state if state is not None else O.basis(qc.num_qubits)
    if qc.num_qubits >= 18:
        re, im = re.copy(), im.copy()
        O.run_inplace(qc, re, im, strategy=O.OR_SIMD_PARALLEL, threads=O.num_cores(), chunks=O.num_cores())
    else:
        re, im = O.run(qc, re, im)
    return re + 1j * im


@pytest.mark.parametrize("n", list(range(8, 21)))
@pytest.mark.parametrize("strategy", [bfy.ExecutionStrategy.GPU, bfy.ExecutionStrategy.GPU_FUSED])
def test_value_encoding_fused_pairs(n, strategy):
    qc = W.encode_value_circuit(n, 4.7)
    fq = FU.fuse_circuit_specialized_pairs(qc)
    assert any(isinstance(t, bfy.FusedPairTransformation) for t in fq.transformations)
    got = run_gpu(fq, strategy)
    assert np.max(np.abs(got - oracle_of(qc))) <= 1e-12


@pytest.mark.parametrize("n,layers", [(13, 6), (16, 4)])
@pytest.mark.parametrize("strategy", [bfy.ExecutionStrategy.GPU, bfy.ExecutionStrategy.GPU_FUSED])
def test_layered_circuit_through_fuse_circuit(n, layers, strategy):
    qc = W.random_layered_circuit(n, layers, seed=n)
    fq = FU.fuse_circuit(qc)
    assert any(isinstance(t, bfy.UnitaryTransformation) and t.m == 2 for t in fq.transformations)
    got = run_gpu(fq, strategy)
    assert np.max(np.abs(got - oracle_of(qc))) <= 1e-12


@pytest.mark.parametrize("fuse", [FU.fuse_circuit, FU.fuse_circuit_specialized_pairs])
def test_fused_qft_from_a_random_state(fuse):
    n = 16
    state = W.random_normal_state(n, 8)
    qc = W.qft_circuit(n)
    got = run_gpu(fuse(qc), bfy.ExecutionStrategy.GPU_FUSED, state=state)
    assert np.max(np.abs(got - oracle_of(qc, state))) <= 1e-12


@pytest.mark.parametrize("n", [12, 17])
def test_complex64_fused_value_encoding(n):
    qc = W.encode_value_circuit(n, 4.7)
    got = run_gpu(FU.fuse_circuit_specialized_pairs(qc), bfy.ExecutionStrategy.GPU_FUSED, dtype="c64")
    exp = oracle_of(qc)
    assert 1 - abs(np.vdot(exp, got)) ** 2 <= 1e-6


def _random_unitary(dim, rng):
    a = rng.normal(size=(dim, dim)) + 1j * rng.normal(size=(dim, dim))
    q, r = np.linalg.qr(a)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _unitary_circuit(n, count, seed):
    """Gates mixed with dense 2- to 5-qubit unitaries, some controlled."""
    rng = np.random.Generator(np.random.PCG64(seed))
    qc = bfy.QuantumCircuit(n)
    for _ in range(count):
        kind = int(rng.integers(0, 6))
        if kind <= 1 or kind >= 4:
            m = 2 + kind if kind <= 1 else kind  # 2, 3, 4 or 5 qubits
            t = int(rng.integers(0, n - m + 1))
            qc.unitary(_random_unitary(1 << m, rng), t, m)
        elif kind == 2:
            t = int(rng.integers(0, n - 1))
            c = int(rng.choice([q for q in range(n) if q < t or q >= t + 2]))
            qc.c_unitary(_random_unitary(4, rng), c, t, 2)
        else:
            qs = [int(x) for x in rng.permutation(n)[:2]]
            qc.u3(qs[0], float(rng.uniform(0, 6)), float(rng.uniform(0, 6)), float(rng.uniform(0, 6)))
            qc.cx(qs[0], qs[1])
    return qc


@pytest.mark.parametrize("n", [9, 13, 16])
@pytest.mark.parametrize("tensor", [True, False])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_dense_unitaries_join_fused_runs(n, tensor, dtype):
    """Dense 2- to 5-qubit unitaries run inside the fused run's tile passes
    (CUDA-core tiles, or multiplied into tensor-core blocks), and the state
    matches the oracle.  A unitary that would be alone in its pass runs as its
    own kernel (the same 2S of traffic), so at most one such pass remains."""
    qc = _unitary_circuit(n, 50, 20 + n)
    state = W.random_normal_state(n, 3)
    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    ctx.gpu_tensor_blocks = tensor
    plan = bfy.plan_stats(qc, ctx, dtype)
    assert plan["other_passes"] <= 1 and plan["tile_passes"] > 0
    if tensor and n >= 12:
        assert plan["block_passes"] > 0
    st = bfy.QuantumState.from_soa(*state, dtype)
    bfy.execute(st, qc, ctx)
    got = st.to_complex()
    st.close()
    exp = oracle_of(qc, state)
    if dtype == "c128":
        assert np.max(np.abs(got - exp)) <= 1e-12
    else:
        assert 1 - abs(np.vdot(exp, got)) ** 2 / (np.vdot(exp, exp).real * np.vdot(got, got).real) <= 1e-6


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_fuse_circuit_layered_runs_in_tile_passes(dtype):
    """fuse_circuit turns a layered circuit's neighbour pairs into 4x4
    unitaries; under GPU_FUSED they stay in the tile passes."""
    n = 18
    qc = W.random_layered_circuit(n, 8, seed=3)
    fq = FU.fuse_circuit(qc)
    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    assert bfy.plan_stats(fq, ctx, dtype)["other_passes"] == 0
    got = run_gpu(fq, bfy.ExecutionStrategy.GPU_FUSED, dtype=dtype)
    exp = oracle_of(qc)
    if dtype == "c128":
        assert np.max(np.abs(got - exp)) <= 1e-12
    else:
        assert 1 - abs(np.vdot(exp, got)) ** 2 <= 1e-6
