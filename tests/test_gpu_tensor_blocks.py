"""complex64 tile passes as 5-qubit blocks on the tensor cores (3xTF32):
parity with the FP64 oracle (infidelity and amplitude error), with the
CUDA-core complex64 path, gates whose controls or diagonal targets lie
outside the tile, passes that fall back to the CUDA-core tile kernel, and the
host-side plan (CPU)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O


def ctx(tensor: bool) -> bfy.ExecContext:
    c = bfy.ExecContext()
    c.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    c.gpu_tensor_blocks = tensor
    return c


def run(qc, re, im, tensor=True, dtype="c64"):
    st = bfy.QuantumState.from_soa(re, im, dtype)
    st.launch_count(reset=True)
    bfy.execute(st, qc, ctx(tensor))
    launches = st.launch_count()
    out = st.to_complex()
    st.close()
    return out, launches


def infidelity(exp, got):
    return 1 - abs(np.vdot(exp, got)) ** 2 / (np.vdot(exp, exp).real * np.vdot(got, got).real)


def check(qc, re, im, tol_inf=1e-6, tol_amp=None):
    got, launches = run(qc, re, im)
    r, i = O.run(qc, re, im)
    exp = r + 1j * i
    assert infidelity(exp, got) <= tol_inf
    if tol_amp is not None:
        assert np.max(np.abs(got - exp)) <= tol_amp
    return got, exp, launches


def random_controlled_circuit(n, count, seed):
    """CX / CCX / CP / CRY / MCX with controls anywhere, U3 on random targets."""
    rng = np.random.Generator(np.random.PCG64(seed))
    qc = bfy.QuantumCircuit(n)
    for _ in range(count):
        kind = int(rng.integers(0, 6))
        qs = [int(x) for x in rng.permutation(n)[:5]]
        if kind == 0:
            qc.cx(qs[0], qs[1])
        elif kind == 1:
            qc.ccx(qs[0], qs[1], qs[2])
        elif kind == 2:
            qc.cp(qs[0], qs[1], float(rng.uniform(0, 2 * math.pi)))
        elif kind == 3:
            qc.cry(qs[0], qs[1], float(rng.uniform(0, 2 * math.pi)))
        elif kind == 4:
            qc.add(qs[:3], qs[3], bfy.X_Gate)
        else:
            a = rng.uniform(0, 2 * math.pi, size=3)
            qc.u3(qs[0], float(a[0]), float(a[1]), float(a[2]))
    return qc


def test_plan_uses_block_passes_only_when_asked():
    qc = W.random_layered_circuit(16, 6, seed=1)
    off = bfy.plan_stats(qc, ctx(False), "c64")
    on = bfy.plan_stats(qc, ctx(True), "c64")
    assert off["block_passes"] == 0 and off["blocks"] == 0
    assert on["block_passes"] > 0 and on["blocks"] >= on["block_passes"]
    assert on["block_passes"] <= on["tile_passes"]


def test_passes_of_diagonal_gates_stay_on_cuda_cores():
    """Controlled phases on many qubit pairs need many blocks but are cheap on
    the CUDA-core tile kernel: such a pass stays there."""
    rng = np.random.Generator(np.random.PCG64(3))
    qc = bfy.QuantumCircuit(16)
    for q in range(16):
        qc.h(q)
    for _ in range(120):
        c, t = (int(x) for x in rng.permutation(12)[:2])
        qc.cp(c, t, float(rng.uniform(0, 2 * math.pi)))
    s = bfy.plan_stats(qc, ctx(True), "c64")
    assert s["tile_passes"] >= 1 and s["block_passes"] < s["tile_passes"]
    q = bfy.plan_stats(W.qft_circuit(20), ctx(True), "c64")
    assert q["block_passes"] < q["tile_passes"]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [12, 13, 16, 18])
def test_random_layered(n):
    qc = W.random_layered_circuit(n, 20, seed=n)
    re, im = O.basis(n)
    got, exp, _ = check(qc, re, im, tol_inf=1e-6)
    # amplitudes ~ 2^-n/2: relative error per amplitude of a few 1e-6 at most
    assert np.max(np.abs(got - exp)) <= 2e-5 * 2 ** (-n / 2) * 10


@pytest.mark.gpu
@pytest.mark.parametrize("n", [12, 15])
def test_qft_from_random_state(n):
    qc = W.qft_circuit(n)
    re, im = W.random_normal_state(n, 5)
    check(qc, re, im, tol_inf=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_controls_and_targets_anywhere(seed):
    n = 16
    qc = random_controlled_circuit(n, 120, seed)
    re, im = W.random_normal_state(n, seed)
    check(qc, re, im, tol_inf=1e-6)


@pytest.mark.gpu
def test_value_encoding_is_the_bit_reversed_basis_state():
    n, v = 14, 9_876
    qc = W.value_encoding_phase_circuit(n, v)
    re, im = O.basis(n)
    got, _ = run(qc, re, im)
    rev = int(format(v, f"0{n}b")[::-1], 2)
    assert abs(got[rev]) ** 2 >= 1 - 1e-6


@pytest.mark.gpu
def test_wide_controls_fall_back_to_the_cuda_core_tile():
    """An MCX with 5 controls spans 6 tile qubits: its pass runs on the
    CUDA-core tile kernel, the others on the tensor cores."""
    n = 14
    qc = W.random_layered_circuit(n, 4, seed=3)
    qc.add([0, 1, 2, 3, 4], 5, bfy.X_Gate)
    for q in range(n):
        qc.h(q)
    re, im = W.random_normal_state(n, 8)
    check(qc, re, im, tol_inf=1e-6)


@pytest.mark.gpu
def test_matches_the_cuda_core_complex64_path():
    n = 16
    qc = W.random_layered_circuit(n, 30, seed=11)
    re, im = O.basis(n)
    a, _ = run(qc, re, im, tensor=True)
    b, _ = run(qc, re, im, tensor=False)
    assert infidelity(b, a) <= 1e-6


@pytest.mark.gpu
def test_small_states_use_the_cuda_core_path():
    n = 10
    qc = W.random_layered_circuit(n, 10, seed=2)
    re, im = O.basis(n)
    check(qc, re, im, tol_inf=1e-6)


@pytest.mark.gpu
def test_complex128_without_tensor_blocks():
    n = 13
    qc = W.random_layered_circuit(n, 8, seed=4)
    re, im = O.basis(n)
    got, _ = run(qc, re, im, tensor=False, dtype="c128")
    r, i = O.run(qc, re, im)
    assert np.max(np.abs(got - (r + 1j * i))) <= 1e-12


@pytest.mark.gpu
def test_state_reuse_after_block_passes():
    """The same state object runs the circuit twice from |0>: equal results."""
    n = 14
    qc = W.random_layered_circuit(n, 6, seed=5)
    st = bfy.QuantumState(n, "c64")
    bfy.execute(st, qc, ctx(True))
    first = st.to_complex()
    st.set_basis(0)
    bfy.execute(st, qc, ctx(True))
    second = st.to_complex()
    st.close()
    assert np.array_equal(first, second)


@pytest.mark.gpu
@pytest.mark.parametrize("da,db", [("c128", "c128"), ("c128", "c64"), ("c64", "c128"), ("c64", "c64")])
def test_inner_product_matches_numpy(da, db):
    n = 15
    ra, ia = W.random_normal_state(n, 1)
    rb, ib = W.random_normal_state(n, 2)
    a = bfy.QuantumState.from_soa(ra, ia, da)
    b = bfy.QuantumState.from_soa(rb, ib, db)
    got = a.inner(b)
    xa, xb = a.to_complex(), b.to_complex()
    a.close()
    b.close()
    exp = np.vdot(xa, xb)
    assert abs(got - exp) <= 1e-13


def test_adjoint_op_array_inverts_on_the_oracle():
    from code_mojo_gb300 import opsarray as OA
    ops = OA.random_layered(8, 6, 3)
    both = OA.OpArray(8, np.concatenate([ops.ops, OA.adjoint(ops).ops]), [])
    r, i = O.run(both, *O.basis(8))
    assert abs(r[0] - 1) <= 1e-12 and np.max(np.abs(r[1:])) <= 1e-12 and np.max(np.abs(i)) <= 1e-12


@pytest.mark.gpu
def test_30q_layered_round_trip_on_tensor_cores():
    """Full size: the 40-layer circuit then its adjoint returns |0> on the
    tensor-core path (complex64, 8 GiB)."""
    from code_mojo_gb300 import opsarray as OA
    n = 30
    ops = OA.random_layered(n, 40, 0)
    assert bfy.plan_stats(ops, ctx(True), "c64")["block_passes"] > 0
    st = bfy.QuantumState(n, "c64")
    bfy.execute(st, ops, ctx(True))
    bfy.execute(st, OA.adjoint(ops), ctx(True))
    top_idx, top_p = st.topk(1)
    st.close()
    assert int(top_idx[0]) == 0 and top_p[0] >= 1 - 1e-5
