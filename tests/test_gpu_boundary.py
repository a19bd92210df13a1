"""Boundary copies of large states: host SoA arrays <-> the device state.

Transfers of at least one staging chunk (2^22 amplitudes) from or to
ordinary pageable arrays go through the library's pinned staging with host
threads; page-locked arrays are copied by DMA directly.  Both must move every
value exactly (complex64 states hold the FP32 rounding of the input)."""
import numpy as np
import pytest

from code_mojo_gb300 import _ffi as F
from code_mojo_gb300 import butterfly as bfy

pytestmark = pytest.mark.gpu


def soa(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.standard_normal(1 << n), rng.standard_normal(1 << n)


@pytest.mark.parametrize("n", [22, 23, 24])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_round_trip_is_exact(n, dtype):
    re, im = soa(n, n)
    st = bfy.QuantumState.from_soa(re, im, dtype)
    gr, gi = st.download()
    st.close()
    if dtype == "c64":
        re, im = re.astype(np.float32).astype(np.float64), im.astype(np.float32).astype(np.float64)
    assert np.array_equal(gr, re) and np.array_equal(gi, im)


def test_ranges_across_chunks():
    n = 24
    re, im = soa(n, 5)
    st = bfy.QuantumState.from_soa(re, im, "c128")
    for off, cnt in [(777, (1 << 22) + 12345), (0, 1 << 23), ((1 << 24) - (1 << 22) - 3, (1 << 22) + 3), (5, 100)]:
        gr, gi = np.empty(cnt), np.empty(cnt)
        F.check(F.lib().bf_state_download_range(st.handle, off, cnt, gr.ctypes.data, gi.ctypes.data))
        assert np.array_equal(gr, re[off:off + cnt]) and np.array_equal(gi, im[off:off + cnt])
    st.close()


def test_page_locked_and_pageable_arrays_agree():
    import torch
    n = 23
    re, im = soa(n, 9)
    cudart = torch.cuda.cudart()
    rc = [int(cudart.cudaHostRegister(a.ctypes.data, a.nbytes, 0)) for a in (re, im)]
    try:
        st = bfy.QuantumState.from_soa(re, im, "c128")
        locked_r, locked_i = np.zeros_like(re), np.zeros_like(im)
        rc2 = [int(cudart.cudaHostRegister(a.ctypes.data, a.nbytes, 0)) for a in (locked_r, locked_i)]
        F.check(F.lib().bf_state_download_soa(st.handle, locked_r.ctypes.data, locked_i.ctypes.data))
        for a, r in zip((locked_r, locked_i), rc2):
            if r == 0:
                cudart.cudaHostUnregister(a.ctypes.data)
        plain_r, plain_i = st.download()
        st.close()
    finally:
        for a, r in zip((re, im), rc):
            if r == 0:
                cudart.cudaHostUnregister(a.ctypes.data)
    assert np.array_equal(locked_r, re) and np.array_equal(locked_i, im)
    assert np.array_equal(plain_r, re) and np.array_equal(plain_i, im)


def test_concurrent_transfers_from_two_threads():
    """Two host threads move two states at once: the library's copy threads
    take one transfer's chunk at a time, and both arrive exactly."""
    import threading
    n = 23
    states = [soa(n, 21), soa(n, 22)]
    out = [None, None]

    def work(k):
        re, im = states[k]
        st = bfy.QuantumState.from_soa(re, im, "c128")
        out[k] = st.download()
        st.close()

    th = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for k in range(2):
        assert np.array_equal(out[k][0], states[k][0]) and np.array_equal(out[k][1], states[k][1])
