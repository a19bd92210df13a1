"""Generates tests/golden/qft_golden.npz: known answers for the gate QFT/IQFT
the reference tests against its classical FFT (tests/test_qft_classical.mojo:
40-103 runs iqft_circuit(...) and its .inverse() on full MSB-first target
lists, with and without the final swap).

The expected vectors come from numpy's FFT and a numpy bit reversal only, not
from the oracle, so they pin the oracle independently:
  QFT  (swap=False) = bitrev(ifft(psi) * sqrt(N))
  QFT  (swap=True)  = bitrev(ifft(bitrev(psi)) * sqrt(N))
  IQFT (swap=False) = fft(bitrev(psi)) / sqrt(N)
  IQFT (swap=True)  = bitrev(fft(bitrev(psi)) / sqrt(N))
plus H^n|0> and the value encoding of an integer v (= |v>).
Run: python tests/golden/make_golden.py
"""
from pathlib import Path

import numpy as np


def bitrev_perm(n):
    idx = np.arange(1 << n, dtype=np.int64)
    r = np.zeros_like(idx)
    for b in range(n):
        r |= ((idx >> b) & 1) << (n - 1 - b)
    return r


def bitrev(v):
    n = int(v.size).bit_length() - 1
    return v[bitrev_perm(n)]


def main():
    out = {}
    for n in (4, 6, 8):
        N = 1 << n
        for seed in (3, 7, 11):
            rng = np.random.Generator(np.random.PCG64(1000 * n + seed))
            psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
            psi /= np.linalg.norm(psi)
            key = f"n{n}_s{seed}"
            out[key + "_in"] = psi
            out[key + "_qft"] = bitrev(np.fft.ifft(psi) * np.sqrt(N))
            out[key + "_qft_swap"] = bitrev(np.fft.ifft(bitrev(psi)) * np.sqrt(N))
            out[key + "_iqft"] = np.fft.fft(bitrev(psi)) / np.sqrt(N)
            out[key + "_iqft_swap"] = bitrev(np.fft.fft(bitrev(psi)) / np.sqrt(N))
    for n in (3, 5, 8):
        out[f"hn_{n}"] = np.full(1 << n, (1 << n) ** -0.5, dtype=np.complex128)
    path = Path(__file__).resolve().parent / "qft_golden.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({len(out)} arrays)")


if __name__ == "__main__":
    main()
