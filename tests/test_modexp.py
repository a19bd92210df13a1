"""Shor's modular exponentiation (apply_modexp / apply_modexp_inverse,
algos/shor.mojo:56-140) and the order-finding circuit: the oracle against a
direct restatement and the closed form on the CPU; the GPU gather
bit-exact against the oracle."""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

CASES = [(4, 4, 7, 15), (3, 4, 2, 15), (5, 5, 4, 21), (4, 6, 11, 35), (6, 5, 5, 31), (2, 3, 3, 8)]


def modexp_reference(re, im, n_exp, n_value, a, N, inverse=False):
    """Direct restatement of apply_modexp's loop."""
    out_re, out_im = np.zeros_like(re), np.zeros_like(im)
    for idx in range(len(re)):
        x, y = idx & ((1 << n_exp) - 1), idx >> n_exp
        y_out = y
        if y < N:
            ax = pow(a, x, N)
            if inverse:
                ax = pow(ax, -1, N)
            y_out = (y * ax) % N
        out_re[x | (y_out << n_exp)] = re[idx]
        out_im[x | (y_out << n_exp)] = im[idx]
    return out_re, out_im


def modexp_only(n_exp, n_value, a, N, inverse=False):
    qc = bfy.QuantumCircuit(n_exp + n_value)
    bfy.mod_exp(qc, n_exp, n_value, a, N)
    return qc.inverse() if inverse else qc


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("inverse", [False, True])
def test_oracle_modexp_matches_the_loop(case, inverse):
    n_exp, n_value, a, N = case
    re, im = W.random_normal_state(n_exp + n_value, 5)
    got = O.run(modexp_only(*case, inverse), re, im)
    exp = modexp_reference(re, im, n_exp, n_value, a, N, inverse)
    assert np.array_equal(got[0], exp[0]) and np.array_equal(got[1], exp[1])


def test_modexp_then_inverse_is_identity():
    case = (5, 5, 4, 21)
    qc = modexp_only(*case)
    qc.transformations += modexp_only(*case, inverse=True).transformations
    re, im = W.random_normal_state(10, 6)
    r, i = O.run(qc, re, im)
    assert np.array_equal(r, re) and np.array_equal(i, im)


@pytest.mark.parametrize("targets,msg", [
    ([4, 4, 7], "MOD_EXP expects 4 parameters: n_exp, n_value, a, N"),
    ([0, 8, 7, 15], "MOD_EXP expects positive register sizes"),
    ([4, 4, 7, 1], "MOD_EXP expects modulus > 1"),
    ([4, 4, 6, 15], "MOD_EXP expects a and modulus to be coprime"),
    ([4, 3, 7, 15], "State size mismatch for MOD_EXP"),
])
def test_modexp_validation_messages(targets, msg):
    qc = bfy.QuantumCircuit(8)
    qc.transformations.append(bfy.ClassicalTransformation("MOD_EXP", targets))
    with pytest.raises(F.BFError) as e:
        bfy.validate(qc)
    assert msg in str(e.value)


def order_from_peak(p_exp, n_exp, N):
    """estimate_order_from_measurement's continued fraction (algos/shor.mojo:190-250)."""
    k = int(np.argmax(p_exp[1:])) + 1
    return Fraction(k, 1 << n_exp).limit_denominator(N).denominator


def textbook_order_finding(n_exp, n_value, a, N):
    """modexp_circuit followed by the inverse QFT over the exponent qubits in
    ascending order with the final swap.  (order_finding_circuit passes the
    exponent qubits to iqft_circuit in descending order, algos/shor.mojo:357,
    which does not concentrate the exponent register on multiples of 2^n/r;
    it is checked for GPU parity only.)"""
    qc = W.modexp_circuit(n_exp, n_value, a, N)
    W.iqft_circuit(qc, list(range(n_exp)), swap=True)
    return qc


def test_order_finding_on_the_oracle_finds_the_order_of_7_mod_15():
    n_exp, n_value, a, N = 6, 4, 7, 15
    qc = textbook_order_finding(n_exp, n_value, a, N)
    r, i = O.run(qc, *O.basis(n_exp + n_value))
    p = (r ** 2 + i ** 2).reshape(1 << n_value, 1 << n_exp).sum(axis=0)  # marginal of the exponent register
    # order 4: the exponent register holds equal peaks at multiples of 2^6 / 4
    peaks = sorted(np.argsort(p)[-4:].tolist())
    assert peaks == [0, 16, 32, 48]
    assert np.allclose(p[peaks], 0.25, atol=1e-12)
    assert order_from_peak(p, n_exp, N) == 4
    assert math.gcd(pow(a, 2) - 1, N) == 3 and math.gcd(pow(a, 2) + 1, N) == 5


@pytest.mark.gpu
# (the last four take the slab-gather form: a value register of at most
# 10 qubits and an exponent register of at least 7)
@pytest.mark.parametrize("case", CASES + [(10, 11, 1234, 2047), (12, 12, 65, 4091), (8, 8, 7, 255),
                                          (9, 7, 5, 127), (12, 10, 77, 1000), (16, 8, 7, 255)])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
@pytest.mark.parametrize("inverse", [False, True])
def test_gpu_modexp_is_bit_exact(case, dtype, inverse):
    n = case[0] + case[1]
    re, im = W.random_normal_state(n, 7)
    if dtype == "c64":
        re, im = re.astype(np.float32).astype(np.float64), im.astype(np.float32).astype(np.float64)
    qc = modexp_only(*case, inverse)
    st = bfy.QuantumState.from_soa(re, im, dtype)
    ctx = bfy.ExecContext()
    ctx.gpu_renormalize = False
    bfy.execute(st, qc, ctx)
    got = st.to_complex()
    st.close()
    r, i = O.run(qc, re, im)
    assert np.array_equal(got.real, r) and np.array_equal(got.imag, i)


@pytest.mark.gpu
@pytest.mark.parametrize("strategy", [bfy.ExecutionStrategy.GPU, bfy.ExecutionStrategy.GPU_FUSED])
@pytest.mark.parametrize("form", ["reference", "textbook"])
def test_gpu_order_finding_matches_the_oracle(strategy, form):
    n_exp, n_value, a, N = 10, 8, 7, 221  # 221 = 13 * 17; the order of 7 is 48
    build = W.order_finding_circuit if form == "reference" else textbook_order_finding
    qc = build(n_exp, n_value, a, N)
    st = bfy.QuantumState(n_exp + n_value)
    ctx = bfy.ExecContext()
    ctx.execution_strategy = strategy
    bfy.execute(st, qc, ctx)
    got = st.to_complex()
    st.close()
    r, i = O.run(qc, *O.basis(n_exp + n_value))
    assert np.max(np.abs(got - (r + 1j * i))) <= 1e-12
    if form == "textbook":
        p = (np.abs(got) ** 2).reshape(1 << n_value, 1 << n_exp).sum(axis=0)
        near = {round(k * (1 << n_exp) / 48) % (1 << n_exp) for k in range(48)}
        assert sum(p[k] for k in near) > 0.4
