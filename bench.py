"""Benchmark: the 30-qubit random layered circuit (complex128, 40 layers of
U3 on every qubit + CX on a random perfect matching, from |0...0>) through
the engine's public API, one GPU per rank (replicas: the workload does not
shard).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step applies the whole circuit once to a state resident in HBM (16 GiB,
larger than L2, so no flush is needed between steps).  `value` is effective
HBM GB/s under the per-gate byte accounting (each dense 1-qubit gate reads and
writes the state once, 2S; each CX touches half of it, S): 3000 S per
circuit.  `roofline` is the pass class with the largest share of the step,
timed with CUDA events around every pass on the state's stream: by default
the complex128 digit block pass (tensor-bound: its bf16 digit products over
the measured bf16 peak, with its 2S of HBM traffic beside it), or the
double-float tile pass (2S per launch) with --no-tensor-blocks.  `e2e` repeats the step through host SoA
buffers (pinned), the upload and the download inside the timed region.
`cpu_baseline` times the restated SIMD_PARALLEL strategy on this host's
cores on a bounded sample of the same circuit.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "30q HBM GB/s vs peak; served circuits/s, p50/p99 ms at fidelity≥1-1e-6"
# DRAM bytes (read + write) per amplitude of one launch, from ncu captures of
# the same kernels on smaller states; traffic grows in proportion to the
# amplitudes a launch processes.  Double-float tile pass: 2.153 GB / 2^26.
TILE_TRAFFIC_BYTES_PER_AMP = 32.08
# complex128 digit block pass (k_tblock_dg), 28 qubits, 4 layers: 4.297 GB
# read + 4.239 GB written / 2^28
DIGIT_TRAFFIC_BYTES_PER_AMP = 31.80
# Tensor work of one complex128 digit block on one 128-row tile (4096
# amplitudes): 26 digit-pair products of 128 x 64 x 64, 2 flops each, for a
# six-digit tile; 20 for a five-digit tile.
DIGIT_FLOPS_PER_AMP_BLOCK = 26 * 2 * 128 * 64 * 64 / 4096
DIGIT_FLOPS_PER_AMP_BLOCK_FIVE = 20 * 2 * 128 * 64 * 64 / 4096
N_QUBITS = 30
LAYERS = 40
SEED = 0


def per_gate_bytes_in_S(qc) -> float:
    """Algorithmic bytes of the per-gate path, in units of the state size S,
    counted from the gates alone (no engine call, so the reference arm never
    loads the engine): a gate reads and writes every amplitude it must
    touch, 2S for a dense or exchanging 1-qubit gate and S for P or Z (only
    the target-1 half changes), each control halving it."""
    from code_mojo_gb300 import butterfly as bfy
    total = 0.0
    for tr in qc.transformations:
        pair = [tr.first, tr.second] if isinstance(tr, bfy.FusedPairTransformation) else [tr]
        for g in pair:
            if isinstance(g, bfy.GateTransformation):
                f = 1.0 if g.gate_info.kind in (bfy.GateKind.P, bfy.GateKind.Z) else 2.0
                total += f / (1 << len(g.controls))
            elif isinstance(g, (bfy.ClassicalTransformation, bfy.QubitReversalTransformation,
                                bfy.UnitaryTransformation, bfy.SwapTransformation)):
                total += 2.0  # a permutation or dense unitary rewrites the whole state once
            else:
                raise ValueError(f"no per-gate byte count for {type(g).__name__}")
    return total


def measured_tensor_peak(sustained: bool) -> tuple[float, str]:
    """Dense bf16 TFLOP/s of this machine's GPUs (cuBLAS), burst or sustained."""
    key = "bf16_tflops_sustained" if sustained else "bf16_tflops"
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())[key]), f"measured {key}"
        except Exception:
            pass
    return (1700.0 if sustained else 1900.0), "fallback bf16"


def roofline_of(times: dict, plan: dict, n: int, S: float, digit_tiles: tuple[int, int] = (0, 0)) -> dict:
    """Roofline of the pass class with the largest share of the timed region
    (CUDA events around each pass on the state's stream).  digit_tiles: the
    five- and six-digit tiles the timed digit passes ran (their digit
    products per block differ)."""
    cls, (count, total_ms) = max(times.items(), key=lambda kv: kv[1][1])
    share = total_ms / sum(t for _, t in times.values())
    avg_ms = total_ms / count
    hbm_peak, hbm_src = measured_peaks()
    hbm = 2 * S / (avg_ms * 1e-3) / 1e9
    if cls == "block_digits":
        # the plan's block count over the timed passes (each step runs the plan once)
        blocks = plan["blocks"] * count / max(1, plan["block_passes"])
        five, six = digit_tiles
        per_amp_block = ((five * DIGIT_FLOPS_PER_AMP_BLOCK_FIVE + six * DIGIT_FLOPS_PER_AMP_BLOCK) / (five + six)
                         if five + six else DIGIT_FLOPS_PER_AMP_BLOCK)
        tflops = per_amp_block * (1 << n) * blocks / (total_ms * 1e-3) / 1e12
        peak, src = measured_tensor_peak(sustained=True)
        traffic = DIGIT_TRAFFIC_BYTES_PER_AMP * (1 << n)
        return {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                "traffic": traffic, "kernel": "bf::k_tblock_dg", "avg_launch_ms": avg_ms,
                "flops_per_launch": per_amp_block * (1 << n) * blocks / count,
                "digit_pairs_per_block": per_amp_block / (2 * 64 * 64 / 32),
                "blocks_per_launch": blocks / count, "share_of_step": share, "launches": count,
                "peak_source": f"{src} (bf16 tensor; digit products are bf16 x bf16 -> fp32)",
                "hbm": {"achieved": hbm, "peak": hbm_peak, "unit": "GB/s", "frac": hbm / hbm_peak,
                        "bytes_per_launch": 2 * S, "peak_source": f"{hbm_src} hbm_gbs"}}
    kernel = {"tile": "bf::k_tile<bf::PolDF, false>", "gate": "bf::k_gate<bf::PolDF>",
              "block_tf32": "bf::k_tblock"}.get(cls, cls)
    traffic = TILE_TRAFFIC_BYTES_PER_AMP * (1 << n) if cls == "tile" else None
    return {"bound": "hbm", "achieved": hbm, "peak": hbm_peak, "unit": "GB/s", "frac": hbm / hbm_peak,
            "traffic": traffic, "kernel": kernel, "bytes_per_launch": 2 * S, "avg_launch_ms": avg_ms,
            "share_of_step": share, "launches": count, "peak_source": f"{hbm_src} hbm_gbs"}


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus: int, backend: str | None = None):
    """Returns (rank, world, local_rank); initialises torch.distributed for N>1
    (NCCL with one GPU per rank; gloo where there is no GPU)."""
    if n_gpus > 1 or "RANK" in os.environ:
        import torch
        import torch.distributed as dist
        rank = int(os.environ.get("RANK", 0))
        world = int(os.environ.get("WORLD_SIZE", 1))
        local = int(os.environ.get("LOCAL_RANK", 0))
        if world > 1 and not dist.is_initialized():
            backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend)
        return rank, world, local
    return 0, 1, 0


def barrier_max(value: float, world: int) -> float:
    """The maximum of `value` over the ranks (each replica's step time)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
def host_state(n: int) -> tuple[np.ndarray, np.ndarray]:
    """|0...0> as host SoA arrays, pages touched before any timing."""
    re = np.empty(1 << n)
    im = np.empty(1 << n)
    re.fill(0.0)
    im.fill(0.0)
    re[0] = 1.0
    return re, im


def cpu_sample(qc, n: int, gates: int, threads: int, state=None) -> dict:
    """Times the restated SIMD_PARALLEL strategy on the first `gates` gates of
    the circuit at full size n (a bounded sample); returns GB/s under the
    per-gate accounting."""
    from code_mojo_gb300 import butterfly as bfy
    from oracle import pyoracle as O
    sample = bfy.QuantumCircuit(n)
    sample.transformations = qc.transformations[:gates]
    bytes_S = per_gate_bytes_in_S(sample)
    S = 16.0 * (1 << n)
    re, im = state if state is not None else host_state(n)
    t0 = time.perf_counter()
    O.run_inplace(sample, re, im, strategy=O.OR_SIMD_PARALLEL, threads=threads, chunks=threads)
    dt = time.perf_counter() - t0
    return {"value": bytes_S * S / dt / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"first {gates} gates of the {n}-qubit {LAYERS}-layer circuit at full size "
                      f"({bytes_S:.0f} S of per-gate traffic in {dt:.2f} s), restated SIMD_PARALLEL strategy",
            "seconds": dt}


def workload_config(world: int) -> dict:
    """The `config` both arms print: the workload, not the engine's settings."""
    return {"workload": f"random layered circuit, {N_QUBITS} qubits, {LAYERS} layers (U3 on every qubit + CX on a "
                        f"random perfect matching), complex128, from |0>",
            "qubits": N_QUBITS, "layers": LAYERS, "seed": SEED, "state_bytes": 16 << N_QUBITS,
            "metric_basis": "per-gate bytes (dense 1-qubit gate 2S, CX S) per circuit / time",
            "l2": "state (16 GiB) larger than L2; no flush", "parallelism": f"replicas x{world}"}


def run_reference(args) -> None:
    rank, world, local = dist_setup(args.gpus)
    if rank != 0:
        return
    from code_mojo_gb300 import workloads as W
    from oracle import pyoracle as O
    qc = W.random_layered_circuit(N_QUBITS, LAYERS, SEED)
    threads = O.num_cores()
    state = host_state(N_QUBITS)
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_sample(qc, N_QUBITS, args.ref_gates, threads, state)
        if i >= args.warmup:
            vals.append(r)
    v = float(np.median([r["value"] for r in vals]))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.median([r["seconds"] for r in vals])) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.gpus),
        "cpu_baseline": {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": "each step: " + vals[0]["sample"]},
        "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_qft_bench(n: int, reps: int) -> dict:
    """The QFT workload: H + n(n-1)/2 CP + a full bit reversal on an N(0,1)
    state (seed 0, unit norm), complex128, fused; CUDA events on the state's
    stream around `reps` applications after 3 warm-up ones.  The 16 MiB state
    of 20 qubits stays in L2, so the bandwidth figures are L2 figures."""
    import torch
    from code_mojo_gb300 import butterfly as bfy
    from code_mojo_gb300 import workloads as W
    qc = W.qft_circuit(n)
    re, im = W.random_normal_state(n, 0)
    st = bfy.QuantumState.from_soa(re, im)
    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    ctx.gpu_sync = False
    stream = torch.cuda.ExternalStream(st.stream_ptr())
    for _ in range(3):
        bfy.execute(st, qc, ctx)
    st.sync()
    st.launch_count(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        bfy.execute(st, qc, ctx)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    launches = st.launch_count() / reps
    st.close()
    plan = bfy.plan_stats(qc, ctx)
    pg = per_gate_bytes_in_S(qc)
    S = 16.0 * (1 << n)
    return {"qubits": n, "gates": len(qc.transformations), "ms_per_circuit": ms, "launches_per_circuit": launches,
            "plan": plan, "per_gate_bytes_in_S": pg, "effective_GB_per_s": pg * S / (ms * 1e-3) / 1e9,
            "fused_GB_per_s": plan["bytes_in_S"] * S / (ms * 1e-3) / 1e9,
            "l2": f"state ({int(S) >> 20} MiB) stays in L2: bandwidths are L2 figures"}


# The reference's published times for this workload (osx-arm64 CPU, median
# of 5 trials x 3 iterations including circuit construction and state
# allocation): benches/results/2026_02_06/execution_strategies_*.csv:17-21
# (GRID_PARALLEL_FUSED, unfused circuit) and benches/results/2026_01_12/
# value_encoding_strategies_qiskit_*.csv:13 (n = 25, GRID_PARALLEL_FUSED).
PUBLISHED_VALUE_ENCODING_MS = {20: 10.72, 22: 83.53, 24: 376.05, 25: 822.66}


def run_value_encoding_bench(sizes, fused_sizes, cpu: bool) -> dict:
    """The reference's value-encoding "full" workload (encode_value_circuit
    with v = 4.7: H on every qubit, P(2 pi v / 2^(j+1)) on qubit j, then the
    MSB-first inverse QFT without swap; benches/bench_execution_strategies.mojo:
    16-34), complex128, from |0...0>.  Per size: the device time of execute
    on a resident state (CUDA events, median of 15 after 3 warm-ups); the
    reference's own method around the public API (circuit construction,
    state creation, execute, synchronisation: wall time, median of 5 trials
    x 3 iterations after one warm-up); and the restated SIMD_PARALLEL
    strategy on this host's cores (median of 3 after one warm-up, circuit
    construction excluded).  `fused_sizes` run the circuit through
    fuse_circuit_specialized_pairs first, as the reference's fused
    benchmark does (benches/bench_value_encoding_strategies_qiskit.mojo:22-39)."""
    import torch
    from code_mojo_gb300 import butterfly as bfy
    from code_mojo_gb300 import fusion as FU
    from code_mojo_gb300 import workloads as W
    v = 4.7
    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    ctx.gpu_sync = False
    out = {"v": v, "dtype": "complex128", "runs": {}}
    cases = [(n, False) for n in sizes] + [(n, True) for n in fused_sizes]
    for n, fused in cases:
        build = (lambda: FU.fuse_circuit_specialized_pairs(W.encode_value_circuit(n, v))) if fused else \
            (lambda: W.encode_value_circuit(n, v))
        qc = build()
        st = bfy.QuantumState(n)
        stream = torch.cuda.ExternalStream(st.stream_ptr())
        dev = []
        for i in range(18):
            st.set_basis(0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            bfy.execute(st, qc, ctx)
            e1.record(stream)
            e1.synchronize()
            if i >= 3:
                dev.append(e0.elapsed_time(e1))
        st.close()
        sctx = ctx.copy()
        sctx.gpu_sync = True

        def ref_method():
            t0 = time.perf_counter()
            c = build()
            s = bfy.QuantumState(n)
            bfy.execute(s, c, sctx)
            s.sync()
            dt = time.perf_counter() - t0
            s.close()
            return dt * 1e3
        ref_method()
        trials = [float(np.median([ref_method() for _ in range(3)])) for _ in range(5)]
        key = f"{n}{'_fused_pairs' if fused else ''}"
        r = {"qubits": n, "fused_pairs": fused, "gates": sum(2 if isinstance(t, bfy.FusedPairTransformation) else 1
                                                             for t in qc.transformations),
             "transformations": len(qc.transformations), "ms": float(np.median(dev)),
             "ms_reference_method": float(np.median(trials)),
             "published_reference_ms": PUBLISHED_VALUE_ENCODING_MS.get(n),
             "plan": bfy.plan_stats(qc, ctx)}
        if r["published_reference_ms"]:
            r["speedup_vs_published"] = r["published_reference_ms"] / r["ms_reference_method"]
        if cpu:
            from oracle import pyoracle as O
            cores = O.num_cores()
            times = []
            for i in range(4):
                re, im = O.basis(n)
                t0 = time.perf_counter()
                O.run_inplace(qc, re, im, strategy=O.OR_SIMD_PARALLEL, threads=cores, chunks=cores)
                if i:
                    times.append((time.perf_counter() - t0) * 1e3)
            r["cpu_port_ms"] = float(np.median(times))
            r["cpu_port_cores"] = cores
        out["runs"][key] = r
    out["published_source"] = ("reference CSVs, osx-arm64 CPU, GRID_PARALLEL_FUSED (benches/results/2026_02_06/"
                               "execution_strategies_*.csv:17-21; n=25: benches/results/2026_01_12/"
                               "value_encoding_strategies_qiskit_*.csv:13)")
    return out


def run_batch_bench(count: int, reps: int, sample: int) -> dict:
    """The batched workload: `count` circuits, qubit counts uniform in [8, 20],
    half random layered (depth 20), half value encodings; one persistent
    launch per run, replayed from a CUDA graph.  complex64 and complex128
    (double-float) runs of the same circuits; the infidelity of the complex64
    outputs against the complex128 ones is checked on a sample."""
    import torch
    from code_mojo_gb300 import batch as B
    from code_mojo_gb300 import opsarray as OA
    circs = OA.batch_mix(count, seed=7)
    rng = np.random.Generator(np.random.PCG64(8))
    out = {"circuits": count, "qubits": "uniform 8..20", "mix": "half random layered depth 20, half value encoding"}
    batches = {}

    def timed(b):
        stream = torch.cuda.ExternalStream(b.stream_ptr())
        b.run()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            b.run(sync=False)
        e1.record(stream)
        e1.synchronize()
        b.sync()
        return e0.elapsed_time(e1) / reps

    for dtype in ("c64", "c128"):
        t0 = time.perf_counter()
        b = B.Batch(circs, dtype=dtype)  # tile widths tuned at creation
        create_s = time.perf_counter() - t0
        ms = timed(b)
        st = b.stats()
        tuning = b.tuning()
        out[dtype] = {"ms_per_batch": ms, "circuits_per_s": count / (ms * 1e-3), "tasks": st["tasks"],
                      "passes": st["passes"], "graph": st["graph"], "state_bytes": st["state_bytes"],
                      "launches_per_batch": 2, "create_s": create_s,
                      "tuned_widths": {str(r["qubits"]): r["width"] for r in tuning if r["chosen"]},
                      "tuning_ms": {f'{r["qubits"]}q_w{r["width"]}': round(r["ms"], 3) for r in tuning}}
        fixed = B.Batch(circs, dtype=dtype, tile_qubits=12)
        fms = timed(fixed)
        fixed.close()
        out[dtype]["fixed_width12_circuits_per_s"] = count / (fms * 1e-3)
        out[dtype]["tuned_over_fixed"] = fms / ms
        batches[dtype] = b
    idx = rng.choice(count, size=min(sample, count), replace=False)
    worst = 0.0
    for c in idx:
        a = batches["c64"].download(int(c))
        r = batches["c128"].download(int(c))
        worst = max(worst, 1 - abs(np.vdot(r, a)) ** 2)
    out["max_infidelity_c64_vs_c128"] = worst
    out["infidelity_sample"] = len(idx)
    out["c64_over_c128_speed"] = out["c64"]["circuits_per_s"] / out["c128"]["circuits_per_s"]
    for b in batches.values():
        b.close()
    return out


def run_serving_bench(rate: float, seconds: float, drain: float, slots: int, capacity_seconds: float = 8.0) -> dict:
    """Poisson arrivals (seeded) of mixed circuits, qubits log-uniform in
    [10, 28] (Grover, value encoding, random layered depth 10..40), each
    returning its top-16 outcomes; complex64 and complex128 runs."""
    from code_mojo_gb300 import serving as SV
    reqs = SV.request_mix(2000, seed=11)
    out = {"rate_per_s": rate, "submit_window_s": seconds, "drain_limit_s": drain, "slots": slots,
           "mix": "Grover / value encoding / random layered, qubits log-uniform 10..28, top-16 returned"}
    for dtype in ("c64", "c128"):
        srv = SV.Server(slots=slots)
        out[dtype] = SV.poisson_run(srv, reqs, rate, seconds, drain, seed=3, dtype=dtype)
        srv.close()
    c64, c128 = out["c64"]["circuits_per_s"], out["c128"]["circuits_per_s"]
    out["c64_over_c128_circuits_per_s"] = c64 / c128 if c128 else None
    # capacity: the same mix with a fixed number of requests in flight
    cap = {"inflight": 2 * slots, "window_s": capacity_seconds}
    if capacity_seconds > 0:
        for dtype in ("c64", "c128"):
            srv = SV.Server(slots=slots)
            cap[dtype] = SV.closed_loop_run(srv, reqs, 2 * slots, capacity_seconds, 60.0, dtype=dtype)
            srv.close()
        a, b = cap["c64"]["circuits_per_s"], cap["c128"]["circuits_per_s"]
        cap["c64_over_c128_circuits_per_s"] = a / b if b else None
        la, lb = cap["c64"]["large"]["per_s"], cap["c128"]["large"]["per_s"]
        cap["c64_over_c128_large_per_s"] = la / lb if lb else None
        # complex64 served results against complex128 ones on a sample of the
        # mix (up to 22 qubits)
        sample = [r for r in reqs if r[1].num_qubits <= 22][:48]
        cap["c64_vs_c128_top16"] = SV.top_probability_gap(sample)
    out["capacity"] = cap
    return out


def run_precision_bench(n_big: int, n_cmp: int, layers: int) -> dict:
    """complex64 at n_big qubits: the layered circuit and a QFT with the gates
    fused into 5-qubit blocks on the tensor cores (3xTF32) against the
    CUDA-core FP32 tile passes; infidelity 1 - |<psi64|psi32>|^2 of the
    tensor-core result against the complex128 (FP64 storage) run of the same
    circuits at n_cmp qubits."""
    from code_mojo_gb300 import butterfly as bfy
    from code_mojo_gb300 import workloads as W

    def ctx(tensor):
        c = bfy.ExecContext()
        c.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
        c.gpu_tensor_blocks = tensor
        c.gpu_tile_qubits = 12
        return c

    def timed(st, qc, c):
        t0 = time.perf_counter()
        bfy.execute(st, qc, c)  # synchronous
        return (time.perf_counter() - t0) * 1e3

    out = {"qubits": n_big, "layers": layers, "state_bytes": 8 << n_big,
           "workload": f"random layered circuit ({layers} layers) then QFT, complex64, from |0>"}
    # warm-up of both kernels on a small state
    w = bfy.QuantumState(16, "c64")
    for t in (True, False):
        bfy.execute(w, W.random_layered_circuit(16, 2, 0), ctx(t))
    w.close()
    qc, qft = W.random_layered_circuit(n_big, layers, SEED), W.qft_circuit(n_big)
    st = bfy.QuantumState(n_big, "c64")
    for name, t in (("tensor_cores", True), ("cuda_cores", False)):
        st.set_basis(0)
        lay = timed(st, qc, ctx(t))
        q = timed(st, qft, ctx(t))
        out[name] = {"layered_ms": lay, "qft_ms": q, "plan_layered": bfy.plan_stats(qc, ctx(t), "c64"),
                     "plan_qft": bfy.plan_stats(qft, ctx(t), "c64")}
    st.close()
    out["tensor_over_cuda_core_speed"] = ((out["cuda_cores"]["layered_ms"] + out["cuda_cores"]["qft_ms"]) /
                                          (out["tensor_cores"]["layered_ms"] + out["tensor_cores"]["qft_ms"]))
    # the tensor-core pass as a roofline: 2S per block pass over the layered run's average pass time
    # (every pass of the layered plan is a block pass or a CUDA-core tile pass of similar length)
    tp = out["tensor_cores"]["plan_layered"]
    passes = max(1, tp["tile_passes"] + tp["gate_kernels"])
    S = float(8 << n_big)
    peak, src = measured_peaks()
    launch_ms = out["tensor_cores"]["layered_ms"] / passes
    blocks = max(1, tp["blocks"])
    out["roofline_k_tblock"] = {
        "bound": "tensor", "kernel": "bf::k_tblock", "avg_launch_ms": launch_ms,
        "hbm": {"achieved": 2 * S / (launch_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                "frac": 2 * S / (launch_ms * 1e-3) / 1e9 / peak, "peak_source": f"{src} hbm_gbs"},
        # 3 TF32 GEMMs of 128 x 64 x 64 per 128-row tile and block: 3 * 2 * 64 * 64 / 32 flop per amplitude
        "tensor": {"achieved": 3 * 2 * 64 * 64 / 32 * (1 << n_big) * blocks / passes / (launch_ms * 1e-3) / 1e12,
                   "unit": "TFLOP/s (TF32)"},
        "blocks_per_pass": blocks / passes}
    # fidelity at n_cmp qubits against complex128
    qc, qft = W.random_layered_circuit(n_cmp, layers, SEED), W.qft_circuit(n_cmp)
    ref = bfy.QuantumState(n_cmp, "c128")
    t128 = timed(ref, qc, ctx(False)) + timed(ref, qft, ctx(False))
    inf = {}
    for name, t in (("tensor_cores", True), ("cuda_cores", False)):
        s32 = bfy.QuantumState(n_cmp, "c64")
        bfy.execute(s32, qc, ctx(t))
        bfy.execute(s32, qft, ctx(t))
        ip = ref.inner(s32)
        inf[name] = 1.0 - abs(ip) ** 2 / (ref.norm2() * s32.norm2())
        s32.close()
    ref.close()
    out["infidelity_vs_complex128"] = {"qubits": n_cmp, **inf}
    out["complex128_ms_at_cmp_qubits"] = t128
    return out


def hbm_figure(plan: dict, n: int, ms_step: float, world: int) -> dict:
    """The metric's HBM reading of the fused step: the bytes its passes must
    move (each tile or block pass reads and writes the state once, 2S) over
    the step time, against the measured copy bandwidth."""
    S = 16.0 * (1 << n)
    peak, src = measured_peaks()
    fused_bytes = plan["bytes_in_S"] * S
    gbs = fused_bytes * world / (ms_step * 1e-3) / 1e9
    return {"fused_bytes_per_step": fused_bytes, "passes_per_step": plan["tile_passes"] + plan["gate_kernels"] +
            plan["other_passes"], "achieved_GBps": gbs, "peak_GBps": peak, "frac_of_peak": gbs / peak / world,
            "peak_source": f"{src} hbm_gbs", "target_frac": 0.70, "target_met": gbs / peak / world >= 0.70}


def summary_of(line: dict) -> dict:
    """The workloads' headline figures in a few keys."""
    def g(d, *path):
        for k in path:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    out = {"circuit30_ms": line["ms_per_step"], "hbm_frac_fused": g(line, "hbm", "frac_of_peak"),
           "digit_pass_ms": g(line, "roofline", "avg_launch_ms"), "e2e_ms": g(line, "e2e", "ms_per_step"),
           "e2e_page_locked_ms": g(line, "e2e", "page_locked", "ms_per_step"),
           "e2e_cold_ms": g(line, "e2e", "cold_first_call_ms"),
           "qft20_ms": g(line, "qft20", "ms_per_circuit")}
    if line.get("value_encoding"):
        out["value_encoding_ms"] = {k: v.get("ms") for k, v in line["value_encoding"].get("runs", {}).items()}
    for dt in ("c64", "c128"):
        out[f"batch_{dt}_circuits_per_s"] = g(line, "batch", dt, "circuits_per_s")
    out["batch_max_infidelity"] = g(line, "batch", "max_infidelity_c64_vs_c128")
    for dt in ("c64", "c128"):
        sv = g(line, "serving", dt) or {}
        out[f"serve_{dt}"] = {k: sv.get(k) for k in ("circuits_per_s", "p50_ms", "p99_ms")} if sv else None
        cap = g(line, "serving", "capacity", dt) or {}
        out[f"capacity_{dt}"] = {k: cap.get(k) for k in ("circuits_per_s", "p50_ms", "p99_ms")} if cap else None
    out["precision_infidelity_32q"] = g(line, "precision", "infidelity_vs_complex128", "tensor_cores")
    out["precision_33q_ms"] = (None if not line.get("precision") else
                               g(line, "precision", "tensor_cores", "layered_ms") +
                               g(line, "precision", "tensor_cores", "qft_ms"))
    return out


def autotune_width(st, qc, candidates) -> tuple[int, dict]:
    """Fusion width: times one layer-block of the circuit at each width and
    keeps the fastest per unit of work."""
    from code_mojo_gb300 import autotune
    return autotune.pick_tile_qubits(st, qc, candidates)


def run_ours(args) -> None:
    rank, world, local = dist_setup(args.gpus)
    import torch
    torch.cuda.set_device(local)
    from code_mojo_gb300 import butterfly as bfy
    from code_mojo_gb300 import workloads as W

    n = N_QUBITS
    S = 16.0 * (1 << n)
    qc = W.random_layered_circuit(n, LAYERS, SEED)
    pg_bytes = per_gate_bytes_in_S(qc) * S
    st = bfy.QuantumState(n)
    stream = torch.cuda.ExternalStream(st.stream_ptr())

    ctx = bfy.ExecContext()
    ctx.execution_strategy = bfy.ExecutionStrategy.GPU_FUSED
    ctx.gpu_tensor_blocks = not args.no_tensor_blocks
    ctx.gpu_sync = False
    if bfy.plan_stats(qc, ctx)["block_passes"] > 0:
        K, tune = 12, "not run: tensor-core block passes fix 12-qubit tiles"
    else:
        K, tune = autotune_width(st, qc, [int(k) for k in args.widths.split(",")])
    ctx.gpu_tile_qubits = K
    plan = bfy.plan_stats(qc, ctx)

    st.set_basis(0)
    for _ in range(args.warmup):
        bfy.execute(st, qc, ctx)
    st.sync()
    barrier(world)
    st.launch_count(reset=True)
    st.digit_tiles(reset=True)
    st.pass_timing(True)
    st.pass_times()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        st.sync()
        e0.record(stream)
        for _ in range(args.steps):
            bfy.execute(st, qc, ctx)
        e1.record(stream)
        e1.synchronize()
    launches = st.launch_count()
    five_tiles, six_tiles = st.digit_tiles()
    pass_times = st.pass_times()
    st.pass_timing(False)
    ms = e0.elapsed_time(e1)
    ms = barrier_max(ms, world)
    ms_step = ms / args.steps
    norm = st.norm2()

    # per-gate path: one circuit (the plain strategy the fused one is compared with)
    per_gate = None
    if args.per_gate_steps > 0:
        pctx = ctx.copy()
        pctx.execution_strategy = bfy.ExecutionStrategy.GPU
        bfy.execute(st, qc, pctx)
        st.sync()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(args.per_gate_steps):
            bfy.execute(st, qc, pctx)
        p1.record(stream)
        p1.synchronize()
        pms = p0.elapsed_time(p1) / args.per_gate_steps
        per_gate = {"ms_per_circuit": pms, "GB_per_s": pg_bytes / (pms * 1e-3) / 1e9,
                    "launches_per_circuit": len(qc.transformations),
                    "frac_of_hbm_peak": pg_bytes / (pms * 1e-3) / 1e9 / measured_peaks()[0]}

    # e2e through the public API with host SoA buffers: the upload of the
    # step's input, the circuit and the download of its result, timed on the
    # host around each step.  The headline uses ordinary pageable arrays (a
    # Mojo List[Float64] is pageable; the library moves large transfers
    # through its pinned staging with host threads); page-locked arrays
    # (registered with cudaHostRegister, copied by DMA directly) and a cold
    # first call on a new state (plan, program upload and copies) are
    # reported beside it.
    e2e = None
    e2e_steps = args.e2e_steps if args.e2e_steps >= 0 else args.steps
    if e2e_steps > 0:
        N = 1 << n
        lib = __import__("code_mojo_gb300._ffi", fromlist=["lib"])
        L = lib.lib()
        ectx = ctx.copy()
        ectx.gpu_sync = True

        def e2e_run(state, hre, him, steps):
            def step():
                lib.check(L.bf_state_upload_soa(state.handle, hre.ctypes.data, him.ctypes.data))
                bfy.execute(state, qc, ectx)
                lib.check(L.bf_state_download_soa(state.handle, hre.ctypes.data, him.ctypes.data))
            times = []
            for _ in range(steps):
                barrier(world)
                t0 = time.perf_counter()
                step()
                times.append(time.perf_counter() - t0)
            return times

        hre, him = host_state(n)
        e2e_run(st, hre, him, 1)  # warm-up
        times = e2e_run(st, hre, him, e2e_steps)
        dt = barrier_max(float(np.mean(times)), world)
        e2e = {"value": pg_bytes * world / dt / 1e9, "unit": "GB/s", "h2d_bytes_per_step": 2 * 8 * N,
               "d2h_bytes_per_step": 2 * 8 * N, "ms_per_step": dt * 1e3, "steps": e2e_steps,
               "host_memory": "pageable (ordinary numpy arrays)", "ms_min": min(times) * 1e3,
               "ms_max": max(times) * 1e3}
        if args.e2e_side_steps > 0:
            cold = bfy.QuantumState(n)
            cold.sync()
            ctimes = e2e_run(cold, hre, him, 1)
            cold.close()
            e2e["cold_first_call_ms"] = ctimes[0] * 1e3
            e2e["cold_first_call"] = ("a new state's first upload + execute (planning and program upload "
                                      "included) + download, pageable host arrays; state creation excluded")
            cudart = torch.cuda.cudart()
            regs = [int(cudart.cudaHostRegister(arr.ctypes.data, arr.nbytes, 0)) for arr in (hre, him)]
            if regs == [0, 0]:
                ltimes = e2e_run(st, hre, him, args.e2e_side_steps)
                ldt = barrier_max(float(np.mean(ltimes)), world)
                e2e["page_locked"] = {"value": pg_bytes * world / ldt / 1e9, "unit": "GB/s",
                                      "ms_per_step": ldt * 1e3, "steps": args.e2e_side_steps,
                                      "ms_min": min(ltimes) * 1e3,
                                      "host_memory": "registered with cudaHostRegister"}
            for arr, rc in zip((hre, him), regs):
                if rc == 0:
                    cudart.cudaHostUnregister(arr.ctypes.data)
        del hre, him

    qft = run_qft_bench(20, 50) if args.qft and rank == 0 else None
    value_enc = (run_value_encoding_bench([20, 22, 24], [25], cpu=args.cpu_gates > 0)
                 if args.value_encoding and rank == 0 else None)
    batch = run_batch_bench(args.batch_count, 3, 256) if args.batch_count > 0 else None
    serving = (run_serving_bench(args.serve_rate, args.serve_seconds, args.serve_seconds, 12, args.capacity_seconds)
               if args.serve_seconds > 0 else None)
    precision = (run_precision_bench(args.precision_qubits, args.precision_qubits - 1, LAYERS)
                 if args.precision_qubits > 0 and rank == 0 else None)

    cpu = None
    if rank == 0 and args.cpu_gates > 0:
        from oracle import pyoracle as O
        cpu = cpu_sample(qc, n, args.cpu_gates, O.num_cores())
        cpu.pop("seconds", None)

    if rank != 0:
        st.close()
        return
    value = pg_bytes * world / (ms_step * 1e-3) / 1e9
    digits = plan["block_passes"] > 0
    arith = ("exact base-256 digit products on bf16 tensor cores (fixed point: one unit, 2^-48 of a power-of-two "
             "scale at least twice the state's norm; a 4096-amplitude tile whose norm is below 2^-9 of the scale "
             "runs five digits, otherwise six, with the same integers; consecutive digit passes hand the state "
             "over as those integers) and double-float tile passes" if digits else "double-float arithmetic")
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fixed48+df64" if digits else "df64", "data": "synthetic",
        "config": workload_config(world),
        "engine": {"arithmetic": f"FP64 storage; {arith}", "tile_qubits": K, "tensor_blocks": digits,
                   "digit_tiles_timed": {"five_digits": five_tiles, "six_digits": six_tiles}},
        "hbm": hbm_figure(plan, n, ms_step, world),
        "gate_passes_per_s": len(qc.transformations) * world / (ms_step * 1e-3),
        "circuits_per_s": world / (ms_step * 1e-3),
        "per_gate_bytes_per_circuit": pg_bytes,
        "fused_plan": plan,
        "roofline": roofline_of(pass_times, plan, n, S, (five_tiles, six_tiles)),
        "pass_times_ms": {k: {"passes": c, "ms": t} for k, (c, t) in pass_times.items()},
        "autotune": tune,
        "per_gate_path": per_gate,
        "gpu_launches": launches,
        "norm_after": norm,
        "norm_after_circuits": args.warmup + args.steps,  # applications of the circuit to the state since |0>
        "clocks": clk.summary(),
        "e2e": e2e,
        "cpu_baseline": cpu,
        "qft20": qft,
        "value_encoding": value_enc,
        "batch": batch,
        "serving": serving,
        "precision": precision,
    }
    line["summary"] = summary_of(line)  # last, so that a tail of the output keeps it
    print(json.dumps(line), flush=True)
    st.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--widths", default="10,11,12,13")
    ap.add_argument("--no-tensor-blocks", action="store_true",
                    help="CUDA-core tile passes only (double-float complex128)")
    ap.add_argument("--per-gate-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=-1, help="-1: as many as --steps")
    ap.add_argument("--e2e-side-steps", "--e2e-pageable-steps", dest="e2e_side_steps", type=int, default=2,
                    help="steps of the page-locked e2e leg (0: skip it and the cold first call)")
    ap.add_argument("--cpu-gates", type=int, default=45)
    ap.add_argument("--ref-gates", type=int, default=45, help="gates per reference-arm step (45: one whole layer)")
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--qft", type=int, default=1, help="time the 20-qubit QFT workload (0: skip)")
    ap.add_argument("--value-encoding", type=int, default=1,
                    help="time the reference's value-encoding workload at 20/22/24 qubits and fused at 25 (0: skip)")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--capacity-seconds", type=float, default=8.0,
                    help="closed-loop serving capacity run per dtype (0: skip)")
    ap.add_argument("--precision-qubits", type=int, default=33,
                    help="complex64 tensor-core vs CUDA-core run at this size (0: skip); fidelity at one qubit less")
    ap.add_argument("--qubits", type=int, default=N_QUBITS,
                    help="state size; anything but 30 is a profiling case, not the benchmark")
    ap.add_argument("--layers", type=int, default=LAYERS,
                    help="circuit depth; anything but 40 is a profiling case, not the benchmark")
    args = ap.parse_args()
    globals()["N_QUBITS"] = args.qubits
    globals()["LAYERS"] = args.layers
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
