"""Grover iterations (classical oracle + full diffuser, repeated) run as one
cooperative loop: parity with the oracle's op-by-op run, launch count, the
closed-form success probability at 20 qubits, and the host-side detection of
the pattern (CPU)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import opsarray as OA
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

TOL128 = 1e-12


def loop_body(n: int, marked: list[int], iters: int) -> OA.OpArray:
    """iters x (classical oracle on `marked`, diffuser over every qubit)."""
    idx = np.array(marked, dtype=np.float64)
    a = np.zeros(2 * iters, dtype=OA.BF_OP)
    a["kind"][0::2] = F.BF_OP_CLASSICAL_ORACLE
    a["data"][0::2] = idx.ctypes.data if len(idx) else 0
    a["nqubits"][0::2] = len(idx)
    a["kind"][1::2] = F.BF_OP_GROVER_DIFFUSER
    return OA.OpArray(n, a, [idx])


@pytest.fixture(params=["df", "f64"])
def c128_math(request, monkeypatch):
    if request.param == "f64":
        monkeypatch.setenv("BFGPU_C128_MATH", "f64")
    else:
        monkeypatch.delenv("BFGPU_C128_MATH", raising=False)
    return request.param


def run(ops, re, im, dtype):
    st = bfy.QuantumState.from_soa(re, im, dtype)
    st.launch_count(reset=True)
    bfy.execute(st, ops)
    launches = st.launch_count()
    out = st.to_complex()
    st.close()
    return out, launches


def test_loop_is_planned_as_one_pass():
    for n in (3, 10, 22):
        s = bfy.plan_stats(loop_body(n, [1], 7))
        assert s["other_passes"] == 1 and s["tile_passes"] == 0 and s["gate_kernels"] == 0
    # a single iteration, or oracles that change, stay per-op
    assert bfy.plan_stats(loop_body(10, [1], 1))["other_passes"] == 2
    a = loop_body(10, [1], 3)
    other = np.array([2.0])
    a.ops["data"][0] = other.ctypes.data
    a.keep.append(other)
    assert bfy.plan_stats(a)["other_passes"] == 3  # pair 0 alone, then a loop of the last two
    # more than eight indices: per-op
    assert bfy.plan_stats(loop_body(10, list(range(9)), 3))["other_passes"] == 6
    # Grover search ops: H^n, then the loop
    s = bfy.plan_stats(OA.grover(12, 5))
    assert s["other_passes"] == 1


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 3, 8, 12, 13, 14, 16, 17, 18])
@pytest.mark.parametrize("marked", [[0], [5, 2, 7], [3, 3], [6, 6, 1]])
def test_loop_matches_oracle_c128(n, marked, c128_math):
    marked = [m % (1 << n) for m in marked]
    iters = 3 if n < 4 else W.grover_iterations(min(n, 12))
    ops = loop_body(n, marked, iters)
    re, im = W.random_normal_state(n, 70 + n)
    got, launches = run(ops, re, im, "c128")
    r, i = O.run(ops, re, im)
    assert np.max(np.abs(got - (r + 1j * i))) <= TOL128
    assert launches == 1


@pytest.mark.gpu
@pytest.mark.parametrize("n", [8, 13, 16, 18, 19])
def test_loop_matches_oracle_c64(n):
    ops = loop_body(n, [n + 1, 3], W.grover_iterations(min(n, 12)))
    re, im = W.random_normal_state(n, 90 + n)
    got, _ = run(ops, re, im, "c64")
    r, i = O.run(ops, re, im)
    exp = r + 1j * i
    assert 1 - abs(np.vdot(exp, got)) ** 2 / (np.vdot(exp, exp).real * np.vdot(got, got).real) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_grover_search_20q_closed_form(dtype):
    """H^20 then the optimal number of iterations: the marked probability is
    sin^2((2r+1) theta) with sin(theta) = 2^-10."""
    n, marked = 20, 777_777
    ops = OA.grover(n, marked)
    r = W.grover_iterations(n)
    st = bfy.QuantumState(n, dtype)
    bfy.execute(st, ops)
    p = st.probabilities(list(range(n)))
    st.close()
    theta = math.asin(2.0 ** (-n / 2))
    exp = math.sin((2 * r + 1) * theta) ** 2
    tol = 1e-10 if dtype == "c128" else 1e-5
    assert abs(p[marked] - exp) <= tol
    rest = (1 - exp) / ((1 << n) - 1)
    others = np.delete(p, marked)
    assert np.max(np.abs(others - rest)) <= (1e-15 if dtype == "c128" else 1e-9)
