"""Contexts used from several host threads at once, as the reference's `kite throughput` runs one
context per pthread (tools/kite.c:65-105): every thread's result is right, on both CUDA engines.
The library shares plans and kernel attributes between contexts behind locks."""
import threading

import pytest

pytestmark = pytest.mark.gpu

CASES = [(9357, 20000, 0x79291CD2F47CE48C, "cuda"), (8191, 25000, 0xD45538E6F07266C6, "cuda"),
         (5, 30000, 0xB7980452FDBC4183, "cuda"), (7, 40001, 0xEB4ADF0EC94C09E6, "cuda"),
         (9357, 20000, 0x79291CD2F47CE48C, "cuda-ntt"), (1365, 45678, 0xEF89209BAE5FF19A, "cuda-ntt")]


def test_concurrent_contexts(lib):
    from ahnum_gb300.kite import CUDA, CUDA_NTT, prp
    results = [None] * len(CASES)

    def run(i, k, n, backend):
        try:
            results[i] = prp(k, n, backend=CUDA_NTT if backend == "cuda-ntt" else CUDA)
        except Exception as e:  # reported below
            results[i] = e

    threads = [threading.Thread(target=run, args=(i, k, n, b)) for i, (k, n, _, b) in enumerate(CASES)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    for (k, n, res, b), r in zip(CASES, results):
        assert not isinstance(r, Exception) and r is not None, (k, n, b, r)
        assert r.rc == 0 and r.res64 == res, f"{b} {k}*2^{n}-1: {r.res64:016X}"
