"""bf_norm2_noalloc: the norm for callers that cannot allocate device memory
(inside stream capture, under a host framework's allocator, or on a path
that cannot take cudaMalloc's implicit synchronisation).  The caller owns the
amplitudes and the output slot; the library's partial sums live in a fixed
512 KiB array built into the library, which caps the input at 2^31
amplitudes.

Each check compares it, through the C ABI, with the allocating entry point
bf_norm2 on the same amplitudes, on two calls in a row (the second call
must not see the first call's leftovers).  This file is collected last so
that a run stopping at its first failure has run every other test first; it
also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import butterfly as bfy
from code_mojo_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-13  # both accumulate in double-float; only the summation order differs


def _torch():
    return pytest.importorskip("torch")


def _device_amps(torch, re, im, dtype):
    z = torch.complex(torch.from_numpy(np.ascontiguousarray(re)), torch.from_numpy(np.ascontiguousarray(im)))
    if dtype == "c64":
        z = z.to(torch.complex64)
    return z.to("cuda")


def _noalloc(torch, d, dtype):
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    code = F.BF_C128 if dtype == "c128" else F.BF_C64
    stream = torch.cuda.current_stream().cuda_stream
    F.check(F.lib().bf_norm2_noalloc(d.data_ptr(), d.numel(), code, out.data_ptr(), stream))
    torch.cuda.current_stream().synchronize()
    return float(out.item())


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_noalloc_matches_bf_norm2_on_two_calls(dtype):
    torch = _torch()
    n = 21
    for call, scale in enumerate((1.0, 1.7)):  # different sums, so stale partials would show
        re, im = W.random_normal_state(n, 40 + call)
        re, im = re * scale, im * scale
        st = bfy.QuantumState.from_soa(re, im, dtype)
        expect = st.norm2()
        st.close()
        got = _noalloc(torch, _device_amps(torch, re, im, dtype), dtype)
        assert abs(got - expect) <= REL_TOL * expect, (call, got, expect)


def test_noalloc_on_a_ragged_count():
    torch = _torch()
    count = (1 << 18) + 12345  # not a whole number of 2^16-amplitude blocks
    rng = np.random.Generator(np.random.PCG64(5))
    re, im = rng.standard_normal(count), rng.standard_normal(count)
    expect = float(np.sum(re * re) + np.sum(im * im))
    for _ in range(2):
        got = _noalloc(torch, _device_amps(torch, re, im, "c128"), "c128")
        assert abs(got - expect) <= REL_TOL * expect


def test_noalloc_rejects_inputs_beyond_its_scratch():
    torch = _torch()
    d = torch.zeros(4, dtype=torch.complex128, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = F.lib().bf_norm2_noalloc(d.data_ptr(), (1 << 31) + 1, F.BF_C128, out.data_ptr(), None)
    assert rc == F.BF_EINVAL
    assert "exceed" in F.last_error()
    rc = F.lib().bf_norm2_noalloc(None, 4, F.BF_C128, out.data_ptr(), None)
    assert rc == F.BF_EINVAL


def test_noalloc_second_call_with_fewer_blocks():
    # the second call covers 3 blocks of partials where the first wrote 32:
    # its finish step must read only its own
    torch = _torch()
    rng = np.random.Generator(np.random.PCG64(9))
    for count in ((1 << 21), (1 << 17) + 5):
        re, im = rng.standard_normal(count), rng.standard_normal(count)
        expect = float(np.sum(re * re) + np.sum(im * im))
        got = _noalloc(torch, _device_amps(torch, re, im, "c128"), "c128")
        assert abs(got - expect) <= REL_TOL * expect, (count, got, expect)


def test_noalloc_rejects_misaligned_pointers_before_launching():
    torch = _torch()
    d = torch.zeros(8, dtype=torch.complex128, device="cuda")
    out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    base, obase = d.data_ptr(), out.data_ptr()
    L = F.lib()
    cases = [(base + 8, F.BF_C128, obase), (base + 4, F.BF_C64, obase), (base, F.BF_C128, obase + 4)]
    for ptr, code, optr in cases:
        assert L.bf_norm2_noalloc(ptr, 4, code, optr, None) == F.BF_EINVAL
        assert "aligned" in F.last_error()
    torch.cuda.synchronize()
    assert float(out[0].item()) == -1.0  # nothing was launched
    # an 8-byte aligned complex64 pointer is fine
    assert L.bf_norm2_noalloc(base + 8, 4, F.BF_C64, obase, None) == F.BF_OK
    torch.cuda.synchronize()
    assert float(out[0].item()) == 0.0


def test_noalloc_inside_a_captured_graph():
    # the use the entry point exists for: a warm-up call outside capture
    # resolves the scratch address, then the call is captured on torch's
    # side stream and replayed with new amplitudes in the same buffer
    torch = _torch()
    n = 19
    d = torch.zeros(1 << n, dtype=torch.complex128, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    L = F.lib()
    F.check(L.bf_norm2_noalloc(d.data_ptr(), d.numel(), F.BF_C128, out.data_ptr(), None))
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        stream = torch.cuda.current_stream().cuda_stream
        F.check(L.bf_norm2_noalloc(d.data_ptr(), d.numel(), F.BF_C128, out.data_ptr(), stream))
    for seed, scale in ((60, 1.0), (61, 0.3)):
        re, im = W.random_normal_state(n, seed)
        re, im = re * scale, im * scale
        d.copy_(_device_amps(torch, re, im, "c128"))
        g.replay()
        torch.cuda.synchronize()
        st = bfy.QuantumState.from_soa(re, im, "c128")
        expect = st.norm2()
        st.close()
        got = float(out.item())
        assert abs(got - expect) <= REL_TOL * expect, (seed, got, expect)
