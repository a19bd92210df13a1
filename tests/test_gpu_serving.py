"""The serving loop: continuous batching over concurrent slots.  Each request's
result is the same when it runs alone and when it runs in the mix, and equals
the oracle's top-16 outcomes."""
import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import opsarray as OA
from code_mojo_gb300 import serving as SV
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def small_mix(count=24, seed=5):
    return SV.request_mix(count, seed=seed, nmin=6, nmax=14)


def run_alone(reqs, dtype):
    srv = SV.Server(slots=1)
    out = {}
    for i, (_, ops) in enumerate(reqs):
        srv.submit(ops, dtype)
        assert srv.wait_idle(60)
        (r,) = srv.poll()
        assert r.status == 0, r.message
        out[i] = r
    srv.close()
    return out


def run_mixed(reqs, dtype, slots=8):
    srv = SV.Server(slots=slots)
    ids = [srv.submit(ops, dtype) for _, ops in reqs]
    assert srv.wait_idle(120)
    res = {r.id: r for r in srv.poll()}
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    return {i: res[rid] for i, rid in enumerate(ids)}, st


@pytest.mark.parametrize("dtype", ["c64", "c128"])
def test_result_is_the_same_alone_and_in_the_mix(dtype):
    # four requests of several milliseconds first, so that the small ones
    # submitted behind them find those slots busy and run on others
    heavy = [("random_layered", OA.random_layered(18, 24, s)) for s in range(4)]
    reqs = heavy + small_mix()
    alone = run_alone(reqs, dtype)
    mixed, st = run_mixed(reqs, dtype)
    tol = 1e-12 if dtype == "c128" else 1e-6
    used_slots = {r.slot for r in mixed.values()}
    assert len(used_slots) > 1  # the requests really ran concurrently
    for i in range(len(reqs)):
        a, m = alone[i], mixed[i]
        # identical inputs and kernels: identical results
        assert a.top_index.tolist() == m.top_index.tolist(), i
        assert np.max(np.abs(a.top_prob - m.top_prob)) <= tol, i


def test_served_results_match_the_oracle():
    reqs = small_mix(12, seed=9)
    mixed, _ = run_mixed(reqs, "c128", slots=4)
    for i, (kind, ops) in enumerate(reqs):
        re, im = O.run(ops, *O.basis(ops.num_qubits))
        p = re * re + im * im
        r = mixed[i]
        # compare probabilities at the served indices, and the served top set
        assert np.max(np.abs(p[r.top_index.astype(np.int64)] - r.top_prob)) <= 1e-12, (i, kind)
        kth = np.sort(p)[::-1][len(r.top_index) - 1]
        assert np.all(p[r.top_index.astype(np.int64)] >= kth - 1e-12), (i, kind)


def test_admission_respects_the_budget():
    n = 14
    budget = 3 * (1 << n) * 8
    srv = SV.Server(slots=8, hbm_budget_bytes=budget)
    for s in range(16):
        srv.submit(OA.random_layered(n, 6, s), "c64")
    assert srv.wait_idle(60)
    st = srv.stats()
    res = srv.poll()
    srv.close()
    assert st["completed"] == 16 and st["peak_bytes"] <= budget
    assert all(r.status == 0 for r in res)


def test_oversize_request_is_refused():
    srv = SV.Server(slots=2, hbm_budget_bytes=1 << 20)
    with pytest.raises(F.BFError) as e:
        srv.submit(OA.random_layered(18, 2, 1), "c128")  # 4 MiB > 1 MiB
    assert e.value.code == F.BF_EBUSY
    srv.close()


def test_wait_idle_is_bounded():
    srv = SV.Server(slots=1)
    srv.submit(OA.grover(20, 12345), "c64")  # ~800 iterations
    assert srv.wait_idle(0.0) is False       # bounded wait returns ETIMEDOUT
    assert srv.wait_idle(120)
    (r,) = srv.poll()
    assert r.status == 0 and int(r.top_index[0]) == 12345 and r.top_prob[0] > 0.99
    srv.close()


def test_large_requests_run_cheapest_first():
    """With one large slot busy, queued large requests start in order of
    2^n * ops, not of arrival."""
    srv = SV.Server(slots=2, large_slots=1, large_cost=1024)
    srv.submit(OA.random_layered(22, 40, 1), "c64")  # occupies the large slot
    reqs = [OA.random_layered(14, 30, 2), OA.random_layered(12, 10, 3), OA.random_layered(13, 20, 4),
            OA.value_encoding(11, 5.0)]
    ids = [srv.submit(ops, "c64") for ops in reqs]
    assert srv.wait_idle(120)
    res = {r.id: r for r in srv.poll()}
    srv.close()
    cost = {rid: (1 << ops.num_qubits) * len(ops) for rid, ops in zip(ids, reqs)}
    assert all(res[rid].status == 0 for rid in ids)
    # queue_s = t_start - t_submit; submissions are microseconds apart, so
    # start order is queue order
    order = sorted(ids, key=lambda rid: res[rid].queue_s)
    assert order == sorted(ids, key=lambda rid: cost[rid])


def test_served_complex64_results_match_the_oracle():
    """complex64 served results against the FP64 oracle: the top-16
    probabilities within 1e-6 of the oracle's at the served indices, and the
    served set is a top-16 set of the oracle's distribution (up to ties
    within that tolerance).  The mix runs Grover searches, value encodings
    and layered circuits of 6..20 qubits on 4 slots at once."""
    reqs = SV.request_mix(16, seed=13, nmin=6, nmax=20)
    mixed, _ = run_mixed(reqs, "c64", slots=4)
    for i, (kind, ops) in enumerate(reqs):
        re, im = O.basis(ops.num_qubits)
        O.run_inplace(ops, re, im, strategy=O.OR_SIMD_PARALLEL, threads=O.num_cores(), chunks=O.num_cores())
        p = re * re + im * im
        r = mixed[i]
        idx = r.top_index.astype(np.int64)
        assert np.max(np.abs(p[idx] - r.top_prob)) <= 1e-6, (i, kind, ops.num_qubits)
        kth = np.sort(p)[::-1][len(idx) - 1]
        assert np.all(p[idx] >= kth - 1e-6), (i, kind)


def test_closed_loop_capacity_run():
    """The capacity run keeps a fixed number of requests in flight: every
    completion in the window is replaced, nothing fails, and the server is
    idle after the drain."""
    reqs = small_mix(32, seed=21)
    srv = SV.Server(slots=4)
    r = SV.closed_loop_run(srv, reqs, inflight=6, duration_s=1.0, drain_s=30.0, dtype="c64")
    st = srv.stats()
    srv.close()
    assert r["failed"] == 0 and r["completed"] > 6 and r["drained_after"]
    assert r["submitted"] >= r["completed"] and r["submitted"] <= r["completed"] + 6 + 64
    assert st["queued"] == 0 and st["running"] == 0
    assert r["circuits_per_s"] > 0 and r["p99_ms"] >= r["p50_ms"] > 0


def test_complex64_and_complex128_served_results_agree():
    gap = SV.top_probability_gap(small_mix(12, seed=23), slots=4)
    assert gap["top_sets_agree"] == 12 and gap["max_top16_prob_gap"] <= 1e-6
