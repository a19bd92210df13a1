"""ctypes loader of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py.  The engine never imports it.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from code_mojo_gb300 import _ffi as F  # noqa: E402  (bf_op layout only; no engine calls)

LIB_PATH = Path(__file__).resolve().parent / "_build" / "liboracle.so"
OR_SCALAR, OR_SIMD_PARALLEL = 0, 3
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} missing: run `make -C oracle`")
        L = C.CDLL(str(LIB_PATH))
        L.or_execute.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(F.bf_op), C.c_int64, C.c_int32,
                                 C.c_int32, C.c_int32, C.c_uint32, C.c_int32, C.c_char_p, C.c_size_t]
        L.or_execute.restype = C.c_int
        L.or_qft_classical.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                       C.c_int32, C.c_char_p, C.c_size_t]
        L.or_qft_classical.restype = C.c_int
        L.or_bit_reverse_indices.argtypes = [C.c_int32, C.c_void_p]
        L.or_bit_reverse_indices.restype = None
        L.or_norm2.argtypes = [C.c_int32, C.c_void_p, C.c_void_p]
        L.or_norm2.restype = C.c_double
        L.or_measure.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int64,
                                 C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_char_p, C.c_size_t]
        L.or_measure.restype = C.c_int
        L.or_topk.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
        L.or_topk.restype = None
        L.or_num_cores.argtypes = []
        L.or_num_cores.restype = C.c_int32
        L.or_fuse.argtypes = [C.c_int32, C.POINTER(F.bf_op), C.c_int64, C.POINTER(F.bf_op), C.c_int64, C.c_void_p,
                              C.c_int64, C.POINTER(C.c_int64), C.c_char_p, C.c_size_t]
        L.or_fuse.restype = C.c_int
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def run(circuit, re: np.ndarray, im: np.ndarray, strategy: int = OR_SCALAR, threads: int = 0, chunks: int = 0,
        specialized: int = 127, validate: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """Runs `circuit` (a butterfly.QuantumCircuit) on copies of (re, im)."""
    re = np.array(re, dtype=np.float64, copy=True)
    im = np.array(im, dtype=np.float64, copy=True)
    n = int(re.size).bit_length() - 1
    arr, cnt, keep = circuit.to_ops()
    err = C.create_string_buffer(512)
    rc = lib().or_execute(n, re.ctypes.data, im.ctypes.data, arr, cnt, strategy, threads, chunks, specialized,
                          1 if validate else 0, err, len(err))
    del keep
    if rc != 0:
        raise OracleError(rc, err.value.decode())
    return re, im


def run_inplace(circuit, re: np.ndarray, im: np.ndarray, strategy: int = OR_SCALAR, threads: int = 0,
                chunks: int = 0) -> None:
    n = int(re.size).bit_length() - 1
    arr, cnt, keep = circuit.to_ops()
    err = C.create_string_buffer(512)
    rc = lib().or_execute(n, re.ctypes.data, im.ctypes.data, arr, cnt, strategy, threads, chunks, 127, 1, err,
                          len(err))
    del keep
    if rc != 0:
        raise OracleError(rc, err.value.decode())


def basis(n: int, idx: int = 0) -> tuple[np.ndarray, np.ndarray]:
    re = np.zeros(1 << n)
    im = np.zeros(1 << n)
    re[idx] = 1.0
    return re, im


def qft_classical(re, im, targets=(), inverse=False, swap=False):
    re = np.array(re, dtype=np.float64, copy=True)
    im = np.array(im, dtype=np.float64, copy=True)
    n = int(re.size).bit_length() - 1
    t = (C.c_int32 * max(1, len(targets)))(*targets)
    err = C.create_string_buffer(512)
    rc = lib().or_qft_classical(n, re.ctypes.data, im.ctypes.data, t, len(targets), int(inverse), int(swap), err,
                                len(err))
    if rc != 0:
        raise OracleError(rc, err.value.decode())
    return re, im


def measure(re, im, targets, values=None, seed=0):
    """apply_measure on copies: returns (outcome, prob, re, im)."""
    re = np.array(re, dtype=np.float64, copy=True)
    im = np.array(im, dtype=np.float64, copy=True)
    n = int(re.size).bit_length() - 1
    t = (C.c_int32 * max(1, len(targets)))(*targets)
    v = None
    if values is not None:
        v = (C.c_int8 * max(1, len(values)))(*[(-1 if x is None else int(x)) for x in values])
    oc, pr = C.c_uint64(), C.c_double()
    err = C.create_string_buffer(512)
    rc = lib().or_measure(n, re.ctypes.data, im.ctypes.data, t, v, len(targets), seed, C.byref(oc), C.byref(pr),
                          err, len(err))
    if rc != 0:
        raise OracleError(rc, err.value.decode())
    return oc.value, pr.value, re, im


def topk(re, im, k):
    n = int(re.size).bit_length() - 1
    idx = np.empty(k, dtype=np.uint64)
    pr = np.empty(k, dtype=np.float64)
    lib().or_topk(n, np.ascontiguousarray(re).ctypes.data, np.ascontiguousarray(im).ctypes.data, k, idx.ctypes.data,
                  pr.ctypes.data)
    return idx, pr


def bit_reverse_indices(n: int) -> np.ndarray:
    out = np.empty(1 << n, dtype=np.uint64)
    lib().or_bit_reverse_indices(n, out.ctypes.data)
    return out


def num_cores() -> int:
    return int(lib().or_num_cores())


FUSE_CIRCUIT, FUSE_SPECIALIZED_PAIRS = 0, 1


def fuse(circuit, mode: int) -> list[dict]:
    """The oracle's restatement of the reference's fusion rewrites applied to
    `circuit`'s records: the rewritten records as dicts (field -> value;
    'data' holds the unitary's complex matrix, row-major)."""
    arr, cnt, keep = circuit.to_ops()
    cap = 2 * cnt + 2
    out = (F.bf_op * cap)()
    mats = np.zeros(32 * cap, dtype=np.float64)
    nout = C.c_int64()
    err = C.create_string_buffer(512)
    rc = lib().or_fuse(mode, arr, cnt, out, cap, mats.ctypes.data, mats.size, C.byref(nout), err, len(err))
    del keep
    if rc != 0:
        raise OracleError(rc, err.value.decode())
    res = []
    for o in out[:nout.value]:
        d = {"kind": o.kind, "gate": o.gate, "target": o.target, "target2": o.target2, "controls": o.controls,
             "ncontrols": o.ncontrols, "flags": o.flags, "arg": o.arg, "mat": list(o.mat)}
        if o.kind in (F.BF_OP_UNITARY, F.BF_OP_CUNITARY):
            dim = 1 << o.target2
            flat = np.ctypeslib.as_array(o.data, shape=(2 * dim * dim,)).copy()
            d["data"] = flat[0::2] + 1j * flat[1::2]
        res.append(d)
    return res
