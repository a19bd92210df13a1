"""Batches of independent circuits in one persistent launch (bf_batch_*)."""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _ffi as F
from .butterfly import QuantumCircuit


class Batch:
    """Runs many small circuits (gate transformations only) from |0...0> in one
    cooperative launch, replayed from a CUDA graph captured at creation."""

    def __init__(self, circuits: Sequence[QuantumCircuit], dtype: str = "c64", tile_qubits: int = 0):
        self._h = C.c_void_p()
        self.dtype = dtype
        self.num_qubits = [c.num_qubits for c in circuits]
        flat = [c.to_ops() for c in circuits]
        nc = len(circuits)
        nq = (C.c_int32 * nc)(*self.num_qubits)
        ptrs = (C.POINTER(F.bf_op) * nc)(*[C.cast(f[0], C.POINTER(F.bf_op)) for f in flat])
        counts = (C.c_int64 * nc)(*[f[1] for f in flat])
        o = F.bf_exec_opts()
        F.check(F.lib().bf_exec_opts_init(C.byref(o)))
        o.tile_qubits = tile_qubits
        code = {"c128": F.BF_C128, "c64": F.BF_C64}[dtype]
        F.check(F.lib().bf_batch_create(nc, nq, ptrs, counts, code, C.byref(o), C.byref(self._h)))
        del flat

    def run(self, sync: bool = True) -> None:
        F.check(F.lib().bf_batch_run(self._h, 1 if sync else 0))

    def sync(self) -> None:
        F.check(F.lib().bf_batch_sync(self._h))

    def download(self, c: int) -> np.ndarray:
        n = self.num_qubits[c]
        re = np.empty(1 << n)
        im = np.empty(1 << n)
        F.check(F.lib().bf_batch_download(self._h, c, re.ctypes.data, im.ctypes.data))
        return re + 1j * im

    def stats(self) -> dict:
        t, p, g = C.c_int64(), C.c_int64(), C.c_int32()
        b, l = C.c_uint64(), C.c_uint64()
        F.check(F.lib().bf_batch_stats(self._h, C.byref(t), C.byref(p), C.byref(b), C.byref(g), C.byref(l)))
        return {"tasks": t.value, "passes": p.value, "state_bytes": b.value, "graph": bool(g.value),
                "launches": l.value}

    def tuning(self) -> list[dict]:
        """The autotuning record: per qubit count, each candidate tile width
        with the time of one run of the sample, and which was chosen."""
        cnt = C.c_int32()
        F.check(F.lib().bf_batch_tuning(self._h, None, None, None, None, 0, C.byref(cnt)))
        m = cnt.value
        q, w, c = (np.zeros(max(m, 1), dtype=np.int32) for _ in range(3))
        ms = np.zeros(max(m, 1), dtype=np.float64)
        F.check(F.lib().bf_batch_tuning(self._h, q.ctypes.data, w.ctypes.data, ms.ctypes.data, c.ctypes.data, m,
                                        C.byref(cnt)))
        return [{"qubits": int(q[r]), "width": int(w[r]), "ms": float(ms[r]), "chosen": bool(c[r])}
                for r in range(m)]

    def stream_ptr(self) -> int:
        s = C.c_void_p()
        F.check(F.lib().bf_batch_stream(self._h, C.byref(s)))
        return s.value or 0

    def close(self) -> None:
        if getattr(self, "_h", None):
            F.lib().bf_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
