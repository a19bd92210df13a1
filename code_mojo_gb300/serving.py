"""Serving: the bf_server_* loop from Python, and the Poisson request stream
used to measure it."""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np

from . import _ffi as F
from . import opsarray as OA


bf_server_opts, bf_result, bf_server_counters = F.bf_server_opts, F.bf_result, F.bf_server_counters


def _lib():
    return F.lib()


@dataclass
class Result:
    id: int
    status: int
    num_qubits: int
    dtype: int
    slot: int
    latency_s: float
    queue_s: float
    top_index: np.ndarray
    top_prob: np.ndarray
    message: str


class Server:
    def __init__(self, slots: int = 12, topk: int = 16, tile_qubits: int = 0, hbm_budget_bytes: int = 0,
                 large_slots: int = 0, large_cost: int = 0):
        o = bf_server_opts(slots, tile_qubits, topk, large_slots, hbm_budget_bytes, large_cost)
        self._h = C.c_void_p()
        F.check(_lib().bf_server_create(C.byref(o), C.byref(self._h)))

    def submit(self, ops: OA.OpArray, dtype: str = "c64") -> int:
        rid = C.c_uint64()
        code = F.BF_C64 if dtype == "c64" else F.BF_C128
        F.check(_lib().bf_server_submit(self._h, ops.num_qubits, code, ops.ops.ctypes.data, len(ops), C.byref(rid)))
        return rid.value

    def submit_serialized(self, blob: bytes, dtype: str = "c64") -> int:
        """Submits a circuit in the binary op-list form (bf_server_submit_serialized)."""
        rid = C.c_uint64()
        code = F.BF_C64 if dtype == "c64" else F.BF_C128
        F.check(_lib().bf_server_submit_serialized(self._h, blob, len(blob), code, C.byref(rid)))
        return rid.value

    def poll(self, max_results: int = 4096) -> list[Result]:
        buf = (bf_result * max_results)()
        cnt = C.c_int32()
        F.check(_lib().bf_server_poll(self._h, buf, max_results, C.byref(cnt)))
        out = []
        for r in buf[:cnt.value]:
            out.append(Result(r.id, r.status, r.num_qubits, r.dtype, r.slot, r.t_done - r.t_submit,
                              r.t_start - r.t_submit, np.array(r.top_index[:r.k], dtype=np.uint64),
                              np.array(r.top_prob[:r.k]), r.message.decode(errors="replace")))
        return out

    def wait_idle(self, timeout_s: float) -> bool:
        rc = _lib().bf_server_wait_idle(self._h, int(timeout_s * 1000))
        if rc == F.BF_ETIMEDOUT:
            return False
        F.check(rc)
        return True

    def stats(self) -> dict:
        c = bf_server_counters()
        F.check(_lib().bf_server_stats(self._h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in bf_server_counters._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib().bf_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# the server's default threshold between small and large requests (2^n * ops)
LARGE_COST = 1 << 28


def request_mix(count: int, seed: int = 0, nmin: int = 10, nmax: int = 28) -> list[tuple[str, OA.OpArray]]:
    """The served mix: qubit counts log-uniform in [nmin, nmax]; kinds Grover
    search (random marked index, floor(pi/4 sqrt(2^n)) iterations), value
    encoding (v uniform in [0, 2^n)) and random layered circuits of depth
    10..40, in equal shares."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        n = min(max(n, nmin), nmax)
        kind = int(rng.integers(0, 3))
        if kind == 0:
            out.append(("grover", OA.grover(n, int(rng.integers(0, 2 ** n)))))
        elif kind == 1:
            out.append(("value_encoding", OA.value_encoding(n, float(rng.uniform(0, 2 ** n)))))
        else:
            out.append(("random_layered", OA.random_layered(n, int(rng.integers(10, 41)), int(rng.integers(0, 2 ** 31)))))
    return out


def poisson_run(server: Server, requests, rate: float, duration_s: float, drain_s: float, seed: int = 0,
                dtype: str = "c64") -> dict:
    """Open-loop Poisson arrivals at `rate` per second for `duration_s`
    seconds (requests taken in order, cycling), then up to `drain_s` seconds
    for the queue to empty.  Reports completed circuits/s over the whole run
    and latency percentiles of the completed requests."""
    rng = np.random.Generator(np.random.PCG64(seed))
    gaps = rng.exponential(1.0 / rate, size=int(rate * duration_s * 2) + 16)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < duration_s]
    t0 = time.perf_counter()
    ids = []
    results = []
    cost = {}
    for i, ta in enumerate(arrivals):
        while True:
            now = time.perf_counter() - t0
            if now >= ta:
                break
            time.sleep(min(0.002, ta - now))
        kind, ops = requests[i % len(requests)]
        ids.append(server.submit(ops, dtype))
        cost[ids[-1]] = (1 << ops.num_qubits) * max(1, len(ops))
        if i % 64 == 0:
            results += server.poll()
    submit_end = time.perf_counter() - t0
    drained = server.wait_idle(drain_s)
    results += server.poll(1 << 16)
    wall = time.perf_counter() - t0
    # every result must belong to a request of this run
    unknown = [r.id for r in results if r.id not in cost]
    if unknown:
        raise RuntimeError(f"{len(unknown)} results with ids this run never submitted, e.g. {unknown[:4]}; "
                           f"{len(ids)} submitted, ids {min(ids)}..{max(ids)}")
    ok = [r for r in results if r.status == 0]
    lat = np.array([r.latency_s for r in ok]) * 1e3
    svc = np.array([r.latency_s - r.queue_s for r in ok]) * 1e3
    nq = np.array([r.num_qubits for r in ok])
    st = server.stats()

    def split(pred):
        sel = [r for r in ok if pred(cost[r.id])]
        la = np.array([r.latency_s for r in sel]) * 1e3
        sub = sum(1 for rid in ids if pred(cost[rid]))
        return {"submitted": sub, "completed": len(sel),
                "p50_ms": float(np.percentile(la, 50)) if len(la) else None,
                "p99_ms": float(np.percentile(la, 99)) if len(la) else None}

    return {"dtype": dtype, "rate_per_s": rate, "submitted": len(ids), "completed": len(ok),
            "failed": len(results) - len(ok), "backlog_at_end": int(st["queued"] + st["running"]),
            "drained": drained, "wall_s": wall, "submit_window_s": submit_end,
            "circuits_per_s": len(ok) / wall if wall > 0 else 0.0,
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "service_p50_ms": float(np.percentile(svc, 50)) if len(svc) else None,
            "service_p99_ms": float(np.percentile(svc, 99)) if len(svc) else None,
            "completed_by_qubits": {int(k): int(v) for k, v in zip(*np.unique(nq, return_counts=True))},
            "peak_state_bytes": int(st["peak_bytes"]),
            "small": split(lambda c: c <= LARGE_COST), "large": split(lambda c: c > LARGE_COST)}


def closed_loop_run(server: Server, requests, inflight: int, duration_s: float, drain_s: float,
                    dtype: str = "c64") -> dict:
    """Capacity of the server on a request mix: `inflight` requests are kept
    submitted at all times (a completed one is replaced by the next of the
    list, cycling) for `duration_s` seconds, then the rest drain (bounded by
    `drain_s`).  Reports the completions per second of the window and the
    latency percentiles of the requests completed in it; with a closed loop
    the queue never grows beyond `inflight`, so these are engine figures,
    not queueing ones."""
    t0 = time.perf_counter()
    cost = {}
    nxt = 0

    def submit_next():
        nonlocal nxt
        kind, ops = requests[nxt % len(requests)]
        nxt += 1
        rid = server.submit(ops, dtype)
        cost[rid] = (1 << ops.num_qubits) * max(1, len(ops))

    for _ in range(inflight):
        submit_next()
    in_window = []
    while time.perf_counter() - t0 < duration_s:
        got = server.poll()
        if not got:
            time.sleep(0.0005)
            continue
        now = time.perf_counter() - t0
        for r in got:
            if r.id not in cost:
                raise RuntimeError(f"result {r.id} was never submitted in this run")
            in_window.append((now, r))
            if now < duration_s:
                submit_next()
    window = time.perf_counter() - t0
    drained = server.wait_idle(drain_s)
    server.poll(1 << 16)
    ok = [r for _, r in in_window if r.status == 0]
    lat = np.array([r.latency_s for r in ok]) * 1e3

    def split(pred):
        la = np.array([r.latency_s for r in ok if pred(cost[r.id])]) * 1e3
        return {"completed": int(len(la)), "per_s": len(la) / window,
                "p50_ms": float(np.percentile(la, 50)) if len(la) else None,
                "p99_ms": float(np.percentile(la, 99)) if len(la) else None}

    nq = np.array([r.num_qubits for r in ok])
    return {"dtype": dtype, "inflight": inflight, "window_s": window, "submitted": nxt, "completed": len(ok),
            "failed": sum(1 for _, r in in_window if r.status != 0), "drained_after": drained,
            "circuits_per_s": len(ok) / window,
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "completed_by_qubits": {int(k): int(v) for k, v in zip(*np.unique(nq, return_counts=True))},
            "small": split(lambda c: c <= LARGE_COST), "large": split(lambda c: c > LARGE_COST)}


def top_probability_gap(reqs, inflight: int = 8, slots: int = 8) -> dict:
    """complex64 against complex128 served results of the same requests: the
    largest difference of the top-16 probabilities at the complex128 result's
    indices, and whether the two top sets agree up to ties within 1e-6."""
    res = {}
    for dtype in ("c64", "c128"):
        srv = Server(slots=slots)
        ids = [srv.submit(ops, dtype) for _, ops in reqs]
        srv.wait_idle(600)
        by = {r.id: r for r in srv.poll(1 << 16)}
        srv.close()
        res[dtype] = [by[i] for i in ids]
    worst, agree = 0.0, 0
    for a, b in zip(res["c64"], res["c128"]):
        pa = dict(zip(a.top_index.tolist(), a.top_prob.tolist()))
        kth = float(b.top_prob[-1])
        same = all(i in pa or float(p) <= kth + 1e-6 for i, p in zip(b.top_index.tolist(), b.top_prob.tolist()))
        agree += int(same)
        for i, p in zip(b.top_index.tolist(), b.top_prob.tolist()):
            if i in pa:
                worst = max(worst, abs(pa[i] - float(p)))
    return {"requests": len(reqs), "max_top16_prob_gap": worst, "top_sets_agree": agree}
