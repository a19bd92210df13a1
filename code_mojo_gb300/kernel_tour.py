"""A tour of the engine's kernels on one state, for profiling and roofline
figures.

  python -m code_mojo_gb300.kernel_tour [--qubits 26] [--dtype c128|c64] [--reps 2]

Each stop runs one operation class through the public API on the same
state (and a small batch), `reps` times, timed with CUDA events on the
state's stream.  A profiler can capture one kernel of the tour by name
(`ncu -k regex:<kernel>`).  The printed JSON lines give, per stop, the
kernel that carries it, its average time, the algorithmic bytes it must
move (in units of the state size S: a gate reads and writes the amplitudes
it changes, a permutation rewrites the state, a reduction reads it) and the
rate those bytes give.  States of 2^26 amplitudes (1 GiB at complex128)
are larger than L2, so the rates are HBM rates.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import butterfly as bfy
from . import opsarray as OA
from . import workloads as W
from .fusion import fuse_circuit


def tour(n: int, dtype: str, reps: int) -> list[dict]:
    import torch

    from .batch import Batch

    st = bfy.QuantumState.from_soa(*W.random_normal_state(n, 1), dtype)
    other = bfy.QuantumState.from_soa(*W.random_normal_state(n, 2), dtype)
    stream = torch.cuda.ExternalStream(st.stream_ptr())
    S = (16 if dtype == "c128" else 8) << n
    per_gate = bfy.ExecContext()
    per_gate.execution_strategy = bfy.ExecutionStrategy.GPU
    fused = bfy.ExecContext()
    fused.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    hi = n - 3  # a high target: pairs 2^(n-3) apart

    def circ(build):
        qc = bfy.QuantumCircuit(n)
        build(qc)
        return qc

    rng = np.random.Generator(np.random.PCG64(5))
    perm = [int(x) for x in rng.permutation(n)]
    u3 = bfy.U3(0.3, 1.1, -0.4)
    stops = [
        ("dense 1-qubit gate (U3)", "k_gate", 2.0, circ(lambda q: q.custom(hi, u3)), per_gate),
        ("Hadamard", "k_gate", 2.0, circ(lambda q: q.h(hi)), per_gate),
        ("phase (P)", "k_gate", 1.0, circ(lambda q: q.p(hi, 0.7)), per_gate),
        ("controlled phase (CP)", "k_gate", 0.5, circ(lambda q: q.cp(2, hi, 0.7)), per_gate),
        ("X", "k_gate", 2.0, circ(lambda q: q.x(hi)), per_gate),
        ("CX", "k_gate", 1.0, circ(lambda q: q.cx(2, hi)), per_gate),
        ("qubit swap (classical)", "k_swap_bits", 1.0,
         circ(lambda q: q.transformations.append(bfy.ClassicalTransformation("SWAP", [1, hi]))), per_gate),
        ("full bit reversal", "k_bitrev_tiles", 2.0, circ(lambda q: bfy.bit_reverse(q)), per_gate),
        ("qubit permutation", "k_permute_tiles", 2.0, circ(lambda q: bfy.permute_qubits(q, perm)), per_gate),
        ("dense 3-qubit unitary", "k_unitary_reg", 2.0,
         circ(lambda q: q.unitary(np.eye(8, dtype=complex) * np.exp(0.3j), hi - 2, 3)), per_gate),
        ("Grover diffuser (classical, all qubits)", "k_diff_sum/k_diff_mean/k_diff_update", 3.0,
         circ(lambda q: bfy.grover_diffuser(q)), per_gate),
        ("modular exponentiation", "k_modexp_slab", 2.0,
         circ(lambda q: q.transformations.append(
             bfy.ClassicalTransformation("MOD_EXP", [n - 8, 8, 7, 255]))), per_gate),
        ("fused layered circuit, 2 layers", "k_tblock_dg / k_tblock / k_tile", None,
         W.random_layered_circuit(n, 2, seed=4), fused),
        ("the same 2 layers after fuse_circuit (4x4 unitaries in the run)", "k_tblock_dg / k_tblock / k_tile", None,
         fuse_circuit(W.random_layered_circuit(n, 2, seed=4)), fused),
    ]
    out = []

    def timed(fn, strm):
        fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(strm)
        for _ in range(reps):
            fn()
        e1.record(strm)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    for name, kernel, bytes_s, qc, ctx in stops:
        ms = timed(lambda: bfy.execute(st, qc, ctx), stream)
        if bytes_s is None:
            bytes_s = bfy.plan_stats(qc, ctx, dtype)["bytes_in_S"]
        out.append({"stop": name, "kernel": kernel, "ms": ms, "bytes_in_S": bytes_s,
                    "GB_per_s": bytes_s * S / (ms * 1e-3) / 1e9})

    # reductions and readout synchronise: timed on the host around the call
    def host_timed(fn):
        fn()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return (time.perf_counter() - t0) / reps * 1e3

    for name, kernel, bytes_s, fn in (
            ("norm", "k_norm2", 1.0, lambda: st.norm2()),
            ("inner product", "k_inner", 2.0, lambda: st.inner(other)),
            ("outcome probabilities of 3 qubits", "k_marginal", 1.0, lambda: st.probabilities([0, 5, hi])),
            ("top-16 outcomes", "k_topk", 1.0, lambda: st.topk(16))):
        ms = host_timed(fn)
        out.append({"stop": name, "kernel": kernel, "ms": ms, "bytes_in_S": bytes_s,
                    "GB_per_s": bytes_s * S / (ms * 1e-3) / 1e9, "timing": "host, includes the readback"})
    # Grover iterations as one loop launch (classical oracle + diffuser pairs)
    iters = 4
    g = OA.grover(n, 12345, iterations=iters)
    g_ops = OA.OpArray(n, g.ops[n:], g.keep)  # without the initial H layer
    ms = timed(lambda: bfy.execute(st, g_ops, per_gate), stream)
    out.append({"stop": f"{iters} Grover iterations", "kernel": "k_grover_loop", "ms": ms,
                "bytes_in_S": 2.0 * iters, "GB_per_s": 2.0 * iters * S / (ms * 1e-3) / 1e9})
    st.close()
    other.close()
    # a batch of small circuits: one persistent launch
    circs = OA.batch_mix(512, seed=9, nmin=10, nmax=14, depth=8)
    b = Batch(circs, dtype=dtype, tile_qubits=10)
    ms = timed(lambda: b.run(sync=False), torch.cuda.ExternalStream(b.stream_ptr()))
    b.sync()
    stt = b.stats()
    out.append({"stop": "batch of 512 circuits (10..14 qubits, depth 8)", "kernel": "k_batch", "ms": ms,
                "tasks": stt["tasks"], "passes": stt["passes"], "state_bytes": stt["state_bytes"],
                "circuits_per_s": 512 / (ms * 1e-3)})
    b.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--qubits", type=int, default=26)
    ap.add_argument("--dtype", default="c128", choices=["c128", "c64"])
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    for r in tour(a.qubits, a.dtype, a.reps):
        print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
