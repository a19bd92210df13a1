"""GPU parity: every kernel path of libbfgpu against the CPU oracle (the
restated SCALAR strategy) on the same seeded inputs.

Tolerances: complex128 results within max|d amp| <= 1e-12 of the oracle
(the bar the reference's own strategies are held to is 1e-10 relative,
bench_execution_strategies.mojo:111-123); permutations bit-exact;
complex64 within infidelity 1 - |<psi64|psi32>|^2 <= 1e-6.
"""
import math
import os

import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
STRATS = [bfy.ExecutionStrategy.GPU, bfy.ExecutionStrategy.GPU_FUSED]


def run_gpu(qc, re, im, strategy=bfy.ExecutionStrategy.GPU_FUSED, K=0, dtype="c128", spec=True):
    st = bfy.QuantumState.from_soa(re, im, dtype)
    ctx = bfy.ExecContext()
    ctx.execution_strategy = strategy
    ctx.gpu_tile_qubits = K
    if not spec:
        for k in list(ctx.__dict__):
            if k.startswith("simd_use_specialized"):
                setattr(ctx, k, False)
    bfy.execute(st, qc, ctx)
    out = st.to_complex()
    st.close()
    return out


def oracle(qc, re, im):
    r, i = O.run(qc, re, im)
    return r + 1j * i


def maxdiff(a, b):
    return float(np.max(np.abs(a - b)))


@pytest.fixture(params=["df", "f64"])
def c128_math(request, monkeypatch):
    """complex128 states compute in double-float by default; BFGPU_C128_MATH=f64
    selects native FP64 arithmetic.  Both must meet the same bar."""
    if request.param == "f64":
        monkeypatch.setenv("BFGPU_C128_MATH", "f64")
    else:
        monkeypatch.delenv("BFGPU_C128_MATH", raising=False)
    return request.param


# ---- every gate kind, controlled and not, at every target class ---------------
GATES = [
    ("h", lambda qc, c, t: qc.add(c, t, bfy.H_Gate)),
    ("x", lambda qc, c, t: qc.add(c, t, bfy.X_Gate)),
    ("y", lambda qc, c, t: qc.add(c, t, bfy.Y_Gate)),
    ("z", lambda qc, c, t: qc.add(c, t, bfy.Z_Gate)),
    ("p", lambda qc, c, t: qc.add(c, t, bfy.P_Gate(0.37))),
    ("rx", lambda qc, c, t: qc.add(c, t, bfy.RX_Gate(1.1))),
    ("ry", lambda qc, c, t: qc.add(c, t, bfy.RY_Gate(-0.8))),
    ("rz", lambda qc, c, t: qc.add(c, t, bfy.RZ_Gate(2.3))),
    ("u3", lambda qc, c, t: qc.add(c, t, bfy.Custom_Gate(bfy.U3(0.3, 1.2, -0.7)))),
]


@pytest.mark.parametrize("name,add", GATES, ids=[g[0] for g in GATES])
@pytest.mark.parametrize("controls,target", [([], 0), ([], 4), ([], 11), ([3], 0), ([0], 11), ([11], 6),
                                             ([1, 9], 5), ([0, 2, 7, 10], 11)])
@pytest.mark.parametrize("strategy", STRATS)
def test_single_gate(name, add, controls, target, strategy, c128_math):
    n = 12
    re, im = W.random_normal_state(n, 17)
    qc = bfy.QuantumCircuit(n)
    add(qc, list(controls), target)
    assert maxdiff(run_gpu(qc, re, im, strategy), oracle(qc, re, im)) <= TOL128


@pytest.mark.parametrize("strategy", STRATS)
def test_generic_kernels_when_specialisation_is_off(strategy):
    n = 10
    re, im = W.random_normal_state(n, 2)
    qc = W.random_layered_circuit(n, 2, 5)
    for q in range(n):
        qc.h(q)
        qc.cp(q, (q + 3) % n, 0.2 * q)
        qc.ry(q, 0.4)
    assert maxdiff(run_gpu(qc, re, im, strategy, spec=False), oracle(qc, re, im)) <= TOL128


# ---- the 20-qubit QFT workload -------------------------------------------------
@pytest.mark.parametrize("strategy", STRATS)
def test_qft20(strategy, c128_math):
    n = 20
    re, im = W.random_normal_state(n, 0)
    qc = W.qft_circuit(n)
    got = run_gpu(qc, re, im, strategy)
    assert maxdiff(got, oracle(qc, re, im)) <= TOL128
    # and the QFT itself: ifft * sqrt(N)
    z = re + 1j * im
    assert maxdiff(got, np.fft.ifft(z) * math.sqrt(1 << n)) <= 1e-12


@pytest.mark.parametrize("n", [8, 10, 11, 16, 21])
def test_full_bit_reversal_is_bit_exact(n):
    re = np.arange(1 << n, dtype=np.float64)
    im = -0.5 * re
    qc = bfy.QuantumCircuit(n)
    bfy.bit_reverse(qc)
    got = run_gpu(qc, re, im)
    exp = oracle(qc, re, im)
    assert np.array_equal(got.real, exp.real) and np.array_equal(got.imag, exp.imag)
    rev = O.bit_reverse_indices(n).astype(np.int64)
    assert np.array_equal(got.real.astype(np.int64), rev)


@pytest.mark.parametrize("build", [
    lambda qc: bfy.bit_reverse(qc, [2, 5, 9, 11]),
    lambda qc: bfy.bit_reverse(qc, [0, 13]),
    lambda qc: bfy.permute_qubits(qc, [13, 0, 5, 1, 12, 2, 3, 4, 6, 7, 8, 9, 10, 11]),
    lambda qc: qc.swap(0, 13),
    lambda qc: qc.swap(4, 5),
    lambda qc: qc.qubit_reversal(),
    lambda qc: qc.qubit_reversal([1, 6, 3, 12]),
    lambda qc: qc.transformations.append(bfy.swap_tr(2, 9)),
])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_permutations_are_bit_exact(build, dtype):
    n = 14
    re = np.arange(1 << n, dtype=np.float64)
    im = re + 0.5
    qc = bfy.QuantumCircuit(n)
    build(qc)
    got = run_gpu(qc, re, im, dtype=dtype)
    exp = oracle(qc, re, im)
    assert np.array_equal(got.real, exp.real) and np.array_equal(got.imag, exp.imag)


# ---- random layered circuits and tile widths ----------------------------------
@pytest.mark.parametrize("strategy", STRATS)
def test_random_layered_16q_40_layers(strategy, c128_math):
    n = 16
    re, im = O.basis(n)
    qc = W.random_layered_circuit(n, 40, seed=1)
    assert maxdiff(run_gpu(qc, re, im, strategy), oracle(qc, re, im)) <= TOL128


@pytest.mark.parametrize("K", [5, 6, 8, 10, 11, 12, 13])
def test_tile_widths(K):
    n = 15
    re, im = W.random_normal_state(n, 3)
    qc = W.random_layered_circuit(n, 6, seed=K)
    qc.transformations += W.qft_circuit(n, with_bit_reversal=False).transformations
    assert maxdiff(run_gpu(qc, re, im, K=K), oracle(qc, re, im)) <= TOL128


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7])
def test_tiny_states(n):
    re, im = W.random_normal_state(n, 1)
    qc = W.random_layered_circuit(n, 3, seed=n)
    bfy.bit_reverse(qc)
    for s in STRATS:
        assert maxdiff(run_gpu(qc, re, im, s), oracle(qc, re, im)) <= TOL128


# ---- value encoding, Grover, fused pairs, unitaries ---------------------------
@pytest.mark.parametrize("strategy", STRATS)
def test_value_encoding_full(strategy):
    for n in (8, 14, 20):
        re, im = O.basis(n)
        qc = W.encode_value_circuit(n, 4.7)
        assert maxdiff(run_gpu(qc, re, im, strategy), oracle(qc, re, im)) <= TOL128


@pytest.mark.parametrize("strategy", STRATS)
def test_grover(strategy):
    n, marked = 10, 677
    re, im = O.basis(n)
    qc = W.grover_circuit(n, marked)
    got = run_gpu(qc, re, im, strategy)
    assert maxdiff(got, oracle(qc, re, im)) <= TOL128
    assert int(np.argmax(np.abs(got))) == marked


@pytest.mark.parametrize("strategy", STRATS)
def test_fused_pairs(strategy):
    n = 12
    re, im = W.random_normal_state(n, 6)
    qc = bfy.QuantumCircuit(n)
    G = bfy.GateTransformation
    qc.append_fused_pair(G([], 6, bfy.H_Gate), G([], 7, bfy.H_Gate))
    qc.append_fused_pair(G([], 9, bfy.H_Gate), G([], 8, bfy.P_Gate(0.3)))
    qc.append_fused_pair(G([], 1, bfy.P_Gate(0.3)), G([], 11, bfy.H_Gate))
    qc.append_fused_pair(G([], 0, bfy.P_Gate(0.7)), G([], 10, bfy.P_Gate(-1.2)))
    qc.append_fused_pair(G([3], 2, bfy.P_Gate(0.5)), G([3], 11, bfy.P_Gate(0.9)))
    qc.append_fused_pair(G([], 4, bfy.RY_Gate(0.5)), G([4], 5, bfy.X_Gate))  # 4x4 path
    assert maxdiff(run_gpu(qc, re, im, strategy), oracle(qc, re, im)) <= TOL128


def random_unitary(dim, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.standard_normal((dim, dim)) + 1j * rng.standard_normal((dim, dim))
    q, r = np.linalg.qr(a)
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("m,target", [(1, 3), (2, 0), (2, 7), (3, 4), (4, 0), (5, 6), (6, 2)])
@pytest.mark.parametrize("controlled", [False, True])
def test_dense_unitaries(m, target, controlled, c128_math):
    n = 13
    re, im = W.random_normal_state(n, m)
    qc = bfy.QuantumCircuit(n)
    u = random_unitary(1 << m, 10 * m + target)
    if controlled:
        ctl = 12 if target + m <= 12 else 0
        qc.c_unitary(u, ctl, target, m)
    else:
        qc.unitary(u, target, m)
    assert maxdiff(run_gpu(qc, re, im, bfy.ExecutionStrategy.GPU), oracle(qc, re, im)) <= TOL128


@pytest.mark.parametrize("m,target", [(1, 9), (2, 0), (2, 3), (3, 1), (3, 10)])
@pytest.mark.parametrize("controlled", [False, True])
def test_dense_unitaries_complex64(m, target, controlled):
    n = 14
    re, im = W.random_normal_state(n, 30 + m)
    qc = bfy.QuantumCircuit(n)
    u = random_unitary(1 << m, 7 * m + target)
    if controlled:
        qc.c_unitary(u, 13 if target + m <= 13 else 0, target, m)
    else:
        qc.unitary(u, target, m)
    z = run_gpu(qc, re, im, bfy.ExecutionStrategy.GPU, dtype="c64")
    exp = oracle(qc, re, im)
    assert 1 - abs(np.vdot(exp, z)) ** 2 / (np.vdot(exp, exp).real * np.vdot(z, z).real) <= 1e-6


# ---- ports of the reference's grid tests --------------------------------------
@pytest.mark.parametrize("n,col_bits", [(10, 5), (12, 6), (14, 7)])
def test_grid_tiling_cases(n, col_bits):
    # tests/test_grid_tiling.mojo: H on the first qubits, then cross-row H/P
    for gate in ("h", "p", "multi"):
        qc = bfy.QuantumCircuit(n)
        for i in range(min(3, n)):
            qc.h(i)
        if gate == "h":
            qc.h(col_bits)
        elif gate == "p":
            qc.p(col_bits, math.pi / 4)
        else:
            qc.h(col_bits)
            qc.p(col_bits + 1, math.pi / 3)
            qc.h(n - 1)
        re, im = O.basis(n)
        for s in STRATS:
            assert maxdiff(run_gpu(qc, re, im, s), oracle(qc, re, im)) <= TOL128


@pytest.mark.parametrize("second", ["hp", "hh", "pp"])
def test_cross_row_fusion_cases(second):
    # tests/test_cross_row_fusion.mojo (n=12, col_bits 6)
    n, cb = 12, 6
    qc = bfy.QuantumCircuit(n)
    for i in range(3):
        qc.h(i)
    if second == "hp":
        qc.h(cb)
        qc.p(cb + 1, math.pi / 4)
    elif second == "hh":
        qc.h(cb)
        qc.h(cb + 1)
    else:
        qc.p(cb, math.pi / 4)
        qc.p(cb + 1, math.pi / 3)
    re, im = O.basis(n)
    for s in STRATS:
        assert maxdiff(run_gpu(qc, re, im, s), oracle(qc, re, im)) <= TOL128


def test_double_float_round_trip_is_unbiased(monkeypatch):
    """P(0) on every qubit, one pass per gate: each pass converts FP64 -> pair
    -> FP64.  The error per element stays below 2^-46 relative and does not
    drift in one direction (the conversions round, they do not truncate)."""
    monkeypatch.delenv("BFGPU_C128_MATH", raising=False)
    n = 14
    re, im = W.random_normal_state(n, 12)
    qc = bfy.QuantumCircuit(n)
    for _ in range(20):
        for q in range(n):
            qc.p(q, 0.0)
    got = run_gpu(qc, re, im, bfy.ExecutionStrategy.GPU)
    z = re + 1j * im
    rel = np.abs(got - z) / np.abs(z)
    assert float(np.max(rel)) < 2.0 ** -40
    bias = np.mean((got.real - z.real) / np.abs(z))
    assert abs(bias) < 2.0 ** -50


# ---- reductions, complex64, errors -------------------------------------------
def test_norm2():
    n = 18
    re, im = W.random_normal_state(n, 9)
    re *= 1.7
    st = bfy.QuantumState.from_soa(re, im)
    assert abs(st.norm2() - O.lib().or_norm2(n, re.ctypes.data, im.ctypes.data)) <= 1e-13
    st.close()


@pytest.mark.parametrize("strategy", STRATS)
def test_complex64_infidelity(strategy):
    n = 16
    re, im = O.basis(n)
    qc = W.random_layered_circuit(n, 20, seed=3)
    got = run_gpu(qc, re, im, strategy, dtype="c64")
    exp = oracle(qc, re, im)
    inf = 1 - abs(np.vdot(exp, got)) ** 2
    assert inf <= 1e-6


def test_execute_raises_reference_messages():
    st = bfy.QuantumState(4)
    qc = bfy.QuantumCircuit(4)
    qc.h(6)
    with pytest.raises(F.BFError, match="Target out of bounds: 6"):
        bfy.execute(st, qc)
    with pytest.raises(F.BFError, match="Circuit qubits mismatch"):
        bfy.execute(st, bfy.QuantumCircuit(5))
    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.SIMD
    with pytest.raises(F.BFError, match="CPU strategy"):
        bfy.execute(st, bfy.QuantumCircuit(4), ctx)
    st.close()


def test_state_reuse_and_launch_count():
    st = bfy.QuantumState(12)
    st.launch_count(reset=True)
    qc = W.qft_circuit(12)
    bfy.execute(st, qc)
    bfy.execute(st, qc.inverse())
    re, im = st.download()
    assert abs(re[0] - 1) < 1e-12 and np.max(np.abs(re[1:])) < 1e-12 and np.max(np.abs(im)) < 1e-12
    assert st.launch_count() > 0
    st.close()


# ---- full size (30 qubits, 16 GiB): size-independent properties ---------------
def adjoint_layered(qc):
    inv = bfy.QuantumCircuit(qc.num_qubits)
    for tr in reversed(qc.transformations):
        g = tr.gate_info
        if g.kind == bfy.GateKind.CUSTOM:
            inv.add(tr.controls, tr.target, bfy.Custom_Gate(g.gate.conj().T))
        else:
            inv.add(tr.controls, tr.target, g)
    return inv


def test_random_layered_30q_round_trip():
    n = 30
    qc = W.random_layered_circuit(n, 40, seed=0)
    st = bfy.QuantumState(n)
    bfy.execute(st, qc)
    assert abs(st.norm2() - 1.0) <= 1e-12
    bfy.execute(st, adjoint_layered(qc))
    re, im = st.download()
    assert abs(re[0] - 1.0) <= 1e-11
    re[0] = 0.0
    assert float(np.max(np.abs(re))) <= 1e-12 and float(np.max(np.abs(im))) <= 1e-12
    st.close()


def test_random_layered_30q_matches_the_oracle():
    """Full size against the oracle itself: two layers of the 30-qubit circuit
    (60 U3 + 30 CX), the oracle's SIMD_PARALLEL port on the host cores (itself
    checked against SCALAR at smaller sizes), compared amplitude by amplitude
    in 64 MiB blocks."""
    n = 30
    qc = W.random_layered_circuit(n, 2, seed=0)
    re, im = O.basis(n)
    O.run_inplace(qc, re, im, strategy=O.OR_SIMD_PARALLEL, threads=O.num_cores(), chunks=O.num_cores())
    st = bfy.QuantumState(n)
    bfy.execute(st, qc)
    blk = 1 << 22
    gr, gi = np.empty(blk), np.empty(blk)
    worst = 0.0
    for off in range(0, 1 << n, blk):
        F.check(F.lib().bf_state_download_range(st.handle, off, blk, gr.ctypes.data, gi.ctypes.data))
        worst = max(worst, float(np.max(np.abs((gr - re[off:off + blk]) + 1j * (gi - im[off:off + blk])))))
    st.close()
    assert worst <= TOL128


def test_random_layered_30q_40_layers_matches_the_oracle(capsys):
    """The benchmarked circuit itself, all 40 layers (1200 U3 + 600 CX, the
    default plan of digit tensor-core passes), against the oracle's
    SIMD_PARALLEL port on every host core, amplitude by amplitude.  The
    worst difference is printed."""
    n = 30
    qc = W.random_layered_circuit(n, 40, seed=0)
    st = bfy.QuantumState(n)
    bfy.execute(st, qc)
    five, six = st.digit_tiles()
    plan = bfy.plan_stats(qc)
    re, im = O.basis(n)
    O.run_inplace(qc, re, im, strategy=O.OR_SIMD_PARALLEL, threads=O.num_cores(), chunks=O.num_cores())
    blk = 1 << 22
    gr, gi = np.empty(blk), np.empty(blk)
    worst = 0.0
    for off in range(0, 1 << n, blk):
        F.check(F.lib().bf_state_download_range(st.handle, off, blk, gr.ctypes.data, gi.ctypes.data))
        worst = max(worst, float(np.max(np.abs((gr - re[off:off + blk]) + 1j * (gi - im[off:off + blk])))))
    st.close()
    with capsys.disabled():
        print(f"\n30-qubit 40-layer circuit ({plan['block_passes']} digit passes, {plan['blocks']} blocks; "
              f"tiles in five / six digits: {five} / {six}): max|d amp| against the oracle = {worst:.3e}")
    assert worst <= TOL128


# ---- measurement and readout (apply_measure, state.mojo:447-553) --------------
@pytest.mark.parametrize("dtype", ["c128", "c64"])
@pytest.mark.parametrize("qubits,values", [([0, 1, 2], None), ([13, 2, 7], None), ([5], None),
                                           ([3, 9, 11, 0], [None, 1, None, 0]), ([], None),
                                           (list(range(12)), None)])
def test_probabilities(dtype, qubits, values):
    n = 14
    re, im = W.random_normal_state(n, 31)
    st = bfy.QuantumState.from_soa(re, im, dtype)
    got = st.probabilities(qubits, values)
    st.close()
    p = re ** 2 + im ** 2
    idx = np.arange(1 << n)
    free = [q for k, q in enumerate(qubits) if values is None or values[k] is None]
    mask = np.ones(1 << n, dtype=bool)
    for k, q in enumerate(qubits):
        if values is not None and values[k] is not None:
            mask &= ((idx >> q) & 1) == values[k]
    outcome = np.zeros(1 << n, dtype=np.int64)
    for j, q in enumerate(free):
        outcome |= ((idx >> q) & 1) << j
    exp = np.bincount(outcome[mask], weights=p[mask], minlength=1 << len(free))
    tol = 1e-14 if dtype == "c128" else 1e-6
    assert np.max(np.abs(got - exp)) <= tol


@pytest.mark.parametrize("targets,values", [([0, 3, 7], None), ([12, 1], [None, True]), (list(range(15)), None),
                                            ([4], None)])
@pytest.mark.parametrize("seed", [1, 77, 2 ** 33 + 5])
def test_measure_matches_oracle(targets, values, seed, c128_math):
    n = 15
    re, im = W.random_normal_state(n, 5)
    st = bfy.QuantumState.from_soa(re, im)
    oc, pr = st.measure(targets, values, seed)
    got = st.to_complex()
    st.close()
    eo, ep, er, ei = O.measure(re, im, targets, values, seed)
    assert oc == eo
    assert abs(pr - ep) <= 1e-14
    assert maxdiff(got, er + 1j * ei) <= TOL128


def test_measure_inside_a_circuit():
    n = 12
    qc = W.random_layered_circuit(n, 3, seed=8)
    bfy.measure(qc, [2, 5, 9], seed=1234)
    qc.transformations += W.random_layered_circuit(n, 2, seed=9).transformations
    bfy.measure(qc, [0, 11], [None, False], seed=99)
    re, im = O.basis(n)
    for s in STRATS:
        assert maxdiff(run_gpu(qc, re, im, s), oracle(qc, re, im)) <= TOL128


def test_measure_zero_probability_raises():
    st = bfy.QuantumState(6)
    with pytest.raises(F.BFError, match="Measurement probability is zero"):
        st.measure([1], [True], 3)
    st.close()


@pytest.mark.parametrize("n,k", [(10, 16), (17, 16), (20, 64), (5, 3)])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_topk(n, k, dtype):
    re, im = W.random_normal_state(n, 40 + n)
    st = bfy.QuantumState.from_soa(re, im, dtype)
    idx, pr = st.topk(k)
    st.close()
    if dtype == "c64":
        re, im = re.astype(np.float32).astype(np.float64), im.astype(np.float32).astype(np.float64)
    ei, ep = O.topk(re, im, k)
    assert idx.tolist() == ei.tolist()
    assert np.max(np.abs(pr - ep) / ep) <= 1e-13  # double-float squares: ~2^-47 relative


def _structured_state(kind, n):
    N = 1 << n
    i = np.arange(N, dtype=np.float64)
    if kind == "uniform":  # every probability equal: the k lowest indices win
        re, im = np.full(N, N ** -0.5), np.zeros(N)
    elif kind == "ramp":  # probabilities rise with the index: every amplitude enters a list
        re, im = np.sqrt(i + 1), np.zeros(N)
    elif kind == "falling":
        re, im = np.zeros(N), -np.sqrt(N - i)
    elif kind == "sparse":  # 5 nonzero amplitudes: the rest of the top k are zeros by index
        re, im = np.zeros(N), np.zeros(N)
        for j, t in enumerate((N - 1, 7, N // 2 + 3, 1, N // 3)):
            re[t], im[t] = 0.1 * (j + 1), -0.05 * j
    else:  # two equal peaks in different CTAs' shares, the rest small
        re, im = np.full(N, 1e-4), np.full(N, -1e-4)
        re[N - 2] = re[3] = 0.5
    s = math.sqrt(float(np.sum(re * re + im * im)))
    return re / s, im / s


@pytest.mark.parametrize("kind", ["uniform", "ramp", "falling", "sparse", "peaks"])
@pytest.mark.parametrize("n,k", [(11, 64), (16, 16), (21, 33), (13, 1)])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_topk_structured(kind, n, k, dtype):
    re, im = _structured_state(kind, n)
    st = bfy.QuantumState.from_soa(re, im, dtype)
    idx, pr = st.topk(k)
    st.close()
    if dtype == "c64":
        re, im = re.astype(np.float32).astype(np.float64), im.astype(np.float32).astype(np.float64)
    ei, ep = O.topk(re, im, k)
    assert idx.tolist() == ei.tolist()
    np.testing.assert_allclose(pr, ep, rtol=1e-13, atol=0)


# ---- classical Grover passes ----------------------------------------------------
@pytest.mark.parametrize("targets", [[], [0, 3, 5], [2, 4, 6, 8, 9, 10, 11, 12, 13], list(range(1, 15)), [14]])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_grover_classical_passes(targets, dtype):
    n = 15
    re, im = W.random_normal_state(n, 60)
    for build in (bfy.grover_diffuser, bfy.grover_inversion_0):
        qc = bfy.QuantumCircuit(n)
        build(qc, targets)
        got = run_gpu(qc, re, im, dtype=dtype)
        exp = oracle(qc, re, im)
        if dtype == "c128":
            assert maxdiff(got, exp) <= TOL128
        else:
            assert 1 - abs(np.vdot(exp, got)) ** 2 <= 1e-6


@pytest.mark.parametrize("strategy", STRATS)
def test_classical_grover_search(strategy):
    n, marked = 12, 3001
    re, im = O.basis(n)
    qc = W.grover_circuit_classical(n, marked)
    got = run_gpu(qc, re, im, strategy)
    assert maxdiff(got, oracle(qc, re, im)) <= TOL128
    assert int(np.argmax(np.abs(got))) == marked
