"""Parity at the benchmark's own configuration.

bench.py times the batched engine with the shipped GB300 four-step shapes
(ahnum_gb300/tuning_gb300.txt), Gerbicz blocks of B = 1000 squarings with a check every M = 250
blocks (first rounds staggered by admission order), and the default block form (the slots in
three parts, each part's pass launches on its own stream, one CUDA graph per block).  These
tests build the batch exactly that way and run full Fermat tests to their RES64:

  * the reference's golden residues at the batched sizes: the 14 primecrunch rows at
    n = 369502..369717 (reference tests/known_residues.csv:14-27) and the known primes
    8243*2^872226-1 and 9001*2^662695-1 (:28-29), in the default form and in the persistent
    kernel's form;
  * 32 of the benchmark's own seeded tests (bench.workload(), one per FFT length first), whose
    RES64s come from the exact integer-NTT engine, itself pinned to GMP and the known residues
    (tests/test_gpu_ntt.py).

Every RES64 must be equal and every round-off below 0.40, the drivers' limit.
"""
import pytest

import bench

pytestmark = pytest.mark.gpu

# reference tests/known_residues.csv:14-29 (k, n, RES64)
PRIMECRUNCH = [
    (9357, 369717, 0xF5FDA01218F20439),
    (9357, 369502, 0xCC259154DD55E913),
    (9357, 369528, 0xC50D87881C4E462E),
    (9357, 369541, 0xCE7F5D87B64DD5E5),
    (9357, 369557, 0xFE6B591A1013CF0B),
    (9357, 369561, 0xE72CD37620A282C7),
    (9357, 369572, 0x5A70E5358FE4B99A),
    (9357, 369584, 0x3B32B08E10EC89C7),
    (9357, 369588, 0xA9BBC7B0F74DDB00),
    (9357, 369606, 0x6A53249346FBA43E),
    (9357, 369620, 0x59E7446E6D1D2E32),
    (9357, 369644, 0xA67076C829354130),
    (9357, 369649, 0x7832CEA658A527FE),
    (9357, 369657, 0xC040400D87FD32DD),
]
KNOWN_PRIMES = [(8243, 872226, 0x1), (9001, 662695, 0x1)]


@pytest.fixture
def bench_shapes(lib):
    """the shipped GB300 shapes, loaded as bench.py loads them; the default shapes afterwards"""
    from ahnum_gb300.tune import load_gb300_tuning, unload_gb300_tuning
    load_gb300_tuning(lib)
    yield
    unload_gb300_tuning(lib)


def _bench_batch():
    from ahnum_gb300 import native
    from ahnum_gb300.kite import Batch
    b = Batch(gerbicz_block=bench.BLOCK, gerbicz_blocks=bench.BLOCKS_PER_CHECK)
    native.load().kc_batch_stagger_checks(b.h, 1)  # as bench.py: first rounds of 1..M blocks
    return b


def _run_to_verdicts(b, tests):
    slots = {}
    for k, n in tests:
        s = b.add_fermat(k, n)
        assert s >= 0, (k, n)
        slots[s] = (k, n)
    b.run()
    out = {}
    for s, (k, n) in slots.items():
        st, r = b.result(s)
        assert st == 1 and r.rc == 0, (k, n, st, r.rc)
        out[(k, n)] = r
    return out


@pytest.mark.parametrize("form", ["three_parts", "persistent"])
def test_bench_form_batch_matches_reference_residues(lib, bench_shapes, monkeypatch, form):
    monkeypatch.delenv("KITE_GB300_BATCH_SPLIT", raising=False)
    if form == "persistent":
        monkeypatch.setenv("KITE_GB300_BATCH_PERSISTENT", "1")
    else:
        monkeypatch.delenv("KITE_GB300_BATCH_PERSISTENT", raising=False)
    rows = PRIMECRUNCH + KNOWN_PRIMES
    with _bench_batch() as b:
        got = _run_to_verdicts(b, [(k, n) for k, n, _ in rows])
    for k, n, res in rows:
        r = got[(k, n)]
        assert r.res64 == res, f"{k}*2^{n}-1: {r.res64:016X} != {res:016X}"
        assert bool(r.is_prp) == (res == 1)
        assert r.fft_len == lib.kc_choose_fft_len(k, n)
        assert 0 < r.maxerr < 0.4, (k, n, r.maxerr)
        assert r.gerbicz_errors == 0 and r.roundoff_retries == 0


def _workload_sample(lib, count=32):
    """bench.workload()'s tests: the first of each FFT length, then the rest in order"""
    tests = bench.workload()
    first, seen = [], set()
    for k, n in tests:
        L = lib.kc_choose_fft_len(k, n)
        if L not in seen:
            seen.add(L)
            first.append((k, n))
    rest = [t for t in tests if t not in first]
    return (first + rest)[:count], seen


def test_bench_workload_matches_exact_ntt_engine(lib, bench_shapes):
    from ahnum_gb300.ntt_group import NttFermatBatch
    tests, lengths = _workload_sample(lib)
    with _bench_batch() as b:
        got = _run_to_verdicts(b, tests)
    with NttFermatBatch(tests, block=bench.BLOCK, blocks_per_check=bench.BLOCKS_PER_CHECK) as nb:
        exact = {(r["k"], r["n"]): r for r in nb.run()}
    assert {got[t].fft_len for t in tests} == lengths
    for t in tests:
        r, x = got[t], exact[t]
        assert r.res64 == x["res64"], f"{t[0]}*2^{t[1]}-1 L={r.fft_len}: {r.res64:016X} != {x['res64']:016X}"
        assert bool(r.is_prp) == bool(x["is_prp"])
        assert 0 < r.maxerr < 0.4, (t, r.fft_len, r.maxerr)
        assert r.gerbicz_errors == 0 and x["gerbicz_errors"] == 0
