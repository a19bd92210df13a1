"""The replica path of bench.py with two ranks over gloo on the CPU: ranks
rendezvous on 127.0.0.1, the step time is the maximum over ranks, and the
reference arm prints from rank 0 only (the other ranks exit without work)."""
from __future__ import annotations

import contextlib
import io
import multiprocessing as mp
import os
import socket
import sys
import types
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    r, w, _ = bench.dist_setup(world, backend="gloo")
    step_ms = 10.0 + 5.0 * r  # rank 1 is the slow replica
    m = bench.barrier_max(step_ms, w)
    bench.barrier(w)
    out = io.StringIO()
    if r != 0:
        # the reference arm on a rank other than 0: returns at once, prints nothing
        args = types.SimpleNamespace(gpus=w, steps=1, warmup=0, ref_gates=1)
        with contextlib.redirect_stdout(out):
            bench.run_reference(args)
    dist.destroy_process_group()
    q.put((r, w, m, out.getvalue()))


def test_two_replicas_take_the_max_step_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1]
    assert all(w == 2 and m == 15.0 for _, w, m, _ in res)
    assert res[1][3] == ""  # rank 1 of the reference arm printed nothing
