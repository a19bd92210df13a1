"""code_mojo_gb300 — a GB300 (sm_103a) statevector engine for Butterfly's
gate-application hot path, reached through the C ABI of libbfgpu.so
(include/bfgpu.h).  `butterfly` mirrors the reference's circuit / execute API
on top of that ABI; `workloads` builds the benchmarked circuits."""
from . import _ffi  # noqa: F401

__all__ = ["butterfly", "workloads"]
