"""ctypes binding of the C ABI in include/bfgpu.h (libbfgpu.so).

This is the binding a Python caller (or a test) uses; a Mojo caller binds the
same symbols through its FFI.  The library is loaded from the package's
_lib/ directory; a missing library is an error, never a silent fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libbfgpu.so"

# status codes
BF_OK, BF_EINVAL, BF_ENOMEM, BF_ECUDA, BF_EUNSUPPORTED, BF_ETIMEDOUT, BF_EBUSY = 0, -1, -2, -3, -4, -5, -6
# dtypes
BF_C128, BF_C64 = 0, 1
# gate kinds (GateKind)
BF_GATE_H, BF_GATE_P, BF_GATE_X, BF_GATE_Y, BF_GATE_Z, BF_GATE_RX, BF_GATE_RY, BF_GATE_RZ, BF_GATE_CUSTOM = range(9)
# op kinds
(BF_OP_GATE, BF_OP_SWAP, BF_OP_QREV, BF_OP_UNITARY, BF_OP_CUNITARY, BF_OP_BITREV, BF_OP_PERMUTE,
 BF_OP_CSWAP, BF_OP_MEASURE, BF_OP_GROVER_DIFFUSER, BF_OP_GROVER_INVERSION0, BF_OP_CLASSICAL_ORACLE,
 BF_OP_MODEXP, BF_OP_MODEXP_INV) = range(14)
BF_OPF_FUSE_WITH_NEXT = 1
BF_STRATEGY_GPU, BF_STRATEGY_GPU_FUSED = 8, 9
BF_SPEC_ALL = 127


class bf_op(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("gate", C.c_int32),
        ("target", C.c_int32),
        ("target2", C.c_int32),
        ("controls", C.c_uint64),
        ("ncontrols", C.c_int32),
        ("flags", C.c_uint32),
        ("arg", C.c_double),
        ("mat", C.c_double * 8),
        ("data", C.POINTER(C.c_double)),
        ("qubits", C.POINTER(C.c_int32)),
        ("nqubits", C.c_int64),
    ]


assert C.sizeof(bf_op) == 128, C.sizeof(bf_op)


class bf_exec_opts(C.Structure):
    _fields_ = [
        ("strategy", C.c_int32),
        ("validate", C.c_int32),
        ("specialized", C.c_uint32),
        ("tile_qubits", C.c_int32),
        ("sync", C.c_int32),
        ("renormalize", C.c_int32),
        ("tensor_blocks", C.c_int32),
        ("plan_dtype", C.c_int32),
    ]


class bf_server_opts(C.Structure):
    _fields_ = [("slots", C.c_int32), ("tile_qubits", C.c_int32), ("topk", C.c_int32), ("large_slots", C.c_int32),
                ("hbm_budget_bytes", C.c_uint64), ("large_cost", C.c_uint64)]


class bf_result(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("num_qubits", C.c_int32), ("dtype", C.c_int32),
                ("slot", C.c_int32), ("k", C.c_int32), ("reserved", C.c_int32), ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_done", C.c_double), ("top_index", C.c_uint64 * 16),
                ("top_prob", C.c_double * 16), ("message", C.c_char * 128)]


class bf_server_counters(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "completed", "failed", "queued", "running", "bytes_in_use",
                                          "peak_bytes", "budget_bytes")]


class BFError(RuntimeError):
    """An error status returned by the engine, with its message."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


_lib = None

# (name, argtypes) of every exported entry point; the CPU test checks that
# the shared library exports exactly these.
SIGNATURES = {
    "bf_exec_opts_init": [C.POINTER(bf_exec_opts)],
    "bf_version": [C.POINTER(C.c_int32)],
    "bf_last_error": [C.c_char_p, C.c_size_t],
    "bf_state_create": [C.c_int32, C.c_int32, C.POINTER(C.c_void_p)],
    "bf_state_destroy": [C.c_void_p],
    "bf_state_info": [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
    "bf_state_set_basis": [C.c_void_p, C.c_uint64],
    "bf_state_upload_soa": [C.c_void_p, C.c_void_p, C.c_void_p],
    "bf_state_download_soa": [C.c_void_p, C.c_void_p, C.c_void_p],
    "bf_state_download_range": [C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p],
    "bf_state_sync": [C.c_void_p],
    "bf_state_stream": [C.c_void_p, C.POINTER(C.c_void_p)],
    "bf_execute": [C.c_void_p, C.POINTER(bf_op), C.c_int64, C.POINTER(bf_exec_opts)],
    "bf_state_launch_count": [C.c_void_p, C.POINTER(C.c_uint64), C.c_int32],
    "bf_state_pass_timing": [C.c_void_p, C.c_int32],
    "bf_state_pass_times": [C.c_void_p, C.c_void_p, C.c_void_p],
    "bf_norm2": [C.c_void_p, C.POINTER(C.c_double)],
    "bf_inner": [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)],
    "bf_probabilities": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p],
    "bf_measure": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_uint64),
                   C.POINTER(C.c_double)],
    "bf_probs_topk": [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p],
    "bf_batch_create": [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(bf_exec_opts),
                        C.POINTER(C.c_void_p)],
    "bf_batch_run": [C.c_void_p, C.c_int32],
    "bf_batch_sync": [C.c_void_p],
    "bf_batch_download": [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p],
    "bf_batch_stats": [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_uint64),
                       C.POINTER(C.c_int32), C.POINTER(C.c_uint64)],
    "bf_batch_stream": [C.c_void_p, C.POINTER(C.c_void_p)],
    "bf_batch_destroy": [C.c_void_p],
    "bf_server_create": [C.POINTER(bf_server_opts), C.POINTER(C.c_void_p)],
    "bf_server_submit": [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_uint64)],
    "bf_server_submit_serialized": [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int32, C.POINTER(C.c_uint64)],
    "bf_qasm3_parse": [C.c_char_p, C.POINTER(C.c_void_p)],
    "bf_ops_serialize": [C.c_int32, C.POINTER(bf_op), C.c_int64, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)],
    "bf_ops_deserialize": [C.c_void_p, C.c_size_t, C.POINTER(C.c_void_p)],
    "bf_oplist_view": [C.c_void_p, C.POINTER(C.POINTER(bf_op)), C.POINTER(C.c_int64), C.POINTER(C.c_int32)],
    "bf_oplist_destroy": [C.c_void_p],
    "bf_server_poll": [C.c_void_p, C.POINTER(bf_result), C.c_int32, C.POINTER(C.c_int32)],
    "bf_server_wait_idle": [C.c_void_p, C.c_int64],
    "bf_server_stats": [C.c_void_p, C.POINTER(bf_server_counters)],
    "bf_server_destroy": [C.c_void_p],
    "bf_norm2_noalloc": [C.c_void_p, C.c_uint64, C.c_int32, C.c_void_p, C.c_void_p],
    "bf_batch_tuning": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                        C.POINTER(C.c_int32)],
    "bf_state_digit_tiles": [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int32],
    "bf_validate": [C.c_int32, C.POINTER(bf_op), C.c_int64],
    "bf_plan_stats": [C.c_int32, C.POINTER(bf_op), C.c_int64, C.POINTER(bf_exec_opts), C.POINTER(C.c_int64),
                      C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_int64),
                      C.POINTER(C.c_int64)],
}


def lib() -> C.CDLL:
    """Loads libbfgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH))
        for name, argtypes in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = argtypes
            fn.restype = C.c_int
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().bf_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != BF_OK:
        raise BFError(rc, last_error())
