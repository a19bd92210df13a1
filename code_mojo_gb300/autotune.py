"""Fusion-width autotuner: times a prefix of the circuit on the caller's state
at each candidate tile width and returns the fastest."""
from __future__ import annotations

import time

from . import butterfly as bfy


def pick_tile_qubits(state: bfy.QuantumState, circuit: bfy.QuantumCircuit, candidates=(10, 11, 12, 13),
                     prefix_gates: int = 180, repeats: int = 2) -> tuple[int, dict]:
    """Returns (best width, {width: seconds for the prefix}).  The state's
    contents are overwritten (the prefix is applied several times)."""
    pre = bfy.QuantumCircuit(circuit.num_qubits)
    pre.transformations = circuit.transformations[:prefix_gates]
    times = {}
    for k in candidates:
        if k > state.num_qubits:
            continue
        ctx = bfy.ExecContext()
        ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
        ctx.gpu_tile_qubits = int(k)
        ctx.gpu_sync = True
        bfy.execute(state, pre, ctx)  # warm: first launch configures the kernel
        best = float("inf")
        for _ in range(repeats):
            t0 = time.perf_counter()
            bfy.execute(state, pre, ctx)
            best = min(best, time.perf_counter() - t0)
        times[int(k)] = best
    if not times:
        return min(state.num_qubits, 11), {}
    return min(times, key=times.get), times
