"""Batches of independent circuits in one persistent launch, checked circuit by
circuit against the FP64 oracle: complex128 within max|d amp| <= 1e-12,
complex64 within infidelity <= 1e-6."""
import numpy as np
import pytest

from code_mojo_gb300 import batch as B
from code_mojo_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def expected(qc):
    r, i = O.run(qc, *O.basis(qc.num_qubits))
    return r + 1j * i


@pytest.mark.parametrize("dtype", ["c64", "c128"])
def test_batch_matches_oracle(dtype):
    circs = W.batch_workload(count=48, seed=3, nmin=4, nmax=16, depth=8)
    b = B.Batch(circs, dtype=dtype)
    st = b.stats()
    assert st["graph"] and st["tasks"] >= len(circs)
    for rep in range(2):  # the graph replays from |0...0> each time
        b.run()
        for c, qc in enumerate(circs):
            got, exp = b.download(c), expected(qc)
            if dtype == "c128":
                assert np.max(np.abs(got - exp)) <= 1e-12, (rep, c)
            else:
                assert 1 - abs(np.vdot(exp, got)) ** 2 <= 1e-6, (rep, c)
    b.close()


def test_batch_with_many_passes_per_circuit():
    # narrow tiles force several dependent passes per circuit
    circs = [W.random_layered_circuit(n, 6, seed=n) for n in (14, 15, 16, 9, 18)]
    b = B.Batch(circs, dtype="c128", tile_qubits=9)
    assert b.stats()["passes"] > len(circs)
    b.run()
    for c, qc in enumerate(circs):
        assert np.max(np.abs(b.download(c) - expected(qc))) <= 1e-12
    b.close()


def test_value_encoding_in_a_batch_lands_on_the_reversed_value():
    vals = [(9, 300), (12, 4095), (10, 1)]
    circs = [W.value_encoding_phase_circuit(n, v) for n, v in vals]
    b = B.Batch(circs, dtype="c64")
    b.run()
    for c, (n, v) in enumerate(vals):
        rev = int(format(v, f"0{n}b")[::-1], 2)
        p = np.abs(b.download(c)) ** 2
        assert int(np.argmax(p)) == rev and p[rev] > 1 - 1e-5
    b.close()


@pytest.mark.parametrize("dtype", ["c64", "c128"])
def test_batch_at_full_spec_matches_the_oracle_per_circuit(dtype):
    """The benchmarked batch itself: 4096 circuits of 8..20 qubits, half
    random layered at depth 20, half value encodings with v uniform in
    [0, 2^n), one persistent launch; a seeded sample of 64 circuits checked
    one by one against the oracle's FP64 run (complex128: max|d amp| <=
    1e-12; complex64: infidelity <= 1e-6)."""
    from code_mojo_gb300 import opsarray as OA
    circs = OA.batch_mix(4096, seed=7)
    b = B.Batch(circs, dtype=dtype)
    b.run()
    rng = np.random.Generator(np.random.PCG64(101 if dtype == "c64" else 102))
    sample = rng.choice(len(circs), size=64, replace=False)
    # the sample covers the whole qubit range and both circuit kinds
    assert max(circs[c].num_qubits for c in sample) >= 19 and len({c % 2 for c in sample}) == 2
    worst = 0.0
    for c in sample:
        ops = circs[int(c)]
        n = ops.num_qubits
        re, im = O.basis(n)
        if n >= 17:
            O.run_inplace(ops, re, im, strategy=O.OR_SIMD_PARALLEL, threads=O.num_cores(), chunks=O.num_cores())
        else:
            re, im = O.run(ops, re, im)
        exp = re + 1j * im
        got = b.download(int(c))
        if dtype == "c128":
            d = float(np.max(np.abs(got - exp)))
            assert d <= 1e-12, (int(c), n, d)
        else:
            d = 1 - abs(np.vdot(exp, got)) ** 2
            assert d <= 1e-6, (int(c), n, d)
        worst = max(worst, d)
    b.close()


def test_batch_autotuning_record_and_result():
    """With tile_qubits = 0 a batch times the candidate tile widths per qubit
    count at creation and keeps the widest within 3% of the fastest; the
    tuned batch still matches the oracle circuit by circuit."""
    circs = W.batch_workload(count=40, seed=9, nmin=6, nmax=13, depth=6)
    b = B.Batch(circs, dtype="c128")
    rows = b.tuning()
    sizes = sorted({qc.num_qubits for qc in circs if qc.num_qubits > 8})
    assert sorted({r["qubits"] for r in rows}) == sizes
    for n in sizes:
        cand = [r for r in rows if r["qubits"] == n]
        assert [r["width"] for r in cand] == list(range(8, min(n, 12) + 1))
        assert sum(r["chosen"] for r in cand) == 1 and all(r["ms"] > 0 for r in cand)
        # the widest width within 3% of the fastest run is kept
        fastest = min(r["ms"] for r in cand)
        keep = max(r["width"] for r in cand if r["ms"] <= 1.03 * fastest)
        assert [r["width"] for r in cand if r["chosen"]] == [keep]
    b.run()
    for c, qc in enumerate(circs):
        assert np.max(np.abs(b.download(c) - expected(qc))) <= 1e-12
    b.close()
    # a fixed width records no tuning
    f = B.Batch(circs[:4], dtype="c64", tile_qubits=10)
    assert f.tuning() == []
    f.close()
