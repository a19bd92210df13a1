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
