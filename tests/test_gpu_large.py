"""Full Fermat tests at production sizes against the reference's golden residues.

The reference's tests/large_fft_cases.csv:4-10 holds seven primecrunch residues (base 3) at
n = 2.29-5.5 million, each confirmed by a certificate on another client, with the FFT length
kite chooses for them.  999*2^4000000-1 (row 8, FFT length 294912) runs through kite_prp on the
CUDA backend in every GPU run; the other six are long (set KITE_GPU_SLOW=1 to run them).  One
row also goes through the served request loop (continuous batching) beside small requests that
arrive while it runs, to show that a verdict at the top of the served n range equals the
golden.
"""
import os

import pytest

pytestmark = pytest.mark.gpu

# reference tests/large_fft_cases.csv:4-10: (k, n, RES64, kite's FFT length)
LARGE = [
    (1021, 2300003, 0x4B048439B12B3423, 163840),
    (6073, 2290815, 0x38C439B2944CD35A, 196608),
    (2009, 3322280, 0x7F4F92B62D7E5381, 262144),
    (6767, 3322174, 0xAD9A7DE7C795812F, 262144),
    (999, 4000000, 0xBBAD057C725281B3, 294912),
    (6119, 4838048, 0xA987B4BF44A5BB74, 393216),
    (4813, 5500155, 0xD6321DD51FA5FB38, 442368),
]
DEFAULT = (999, 4000000)
SLOW = os.environ.get("KITE_GPU_SLOW") == "1"


def _check(lib, k, n, res, L):
    from ahnum_gb300.kite import prp
    assert lib.kc_choose_fft_len(k, n) == L
    r = prp(k, n)
    assert r.rc == 0, r.rc
    assert r.fft_len == L
    assert r.res64 == res, f"{k}*2^{n}-1: {r.res64:016X} != {res:016X}"
    assert not r.is_prp
    assert r.maxerr < 0.4


@pytest.mark.parametrize("k,n,res,L", [c for c in LARGE if c[:2] == DEFAULT])
def test_large_fermat_matches_golden(lib, k, n, res, L):
    _check(lib, k, n, res, L)


@pytest.mark.skipif(not SLOW, reason="long: KITE_GPU_SLOW=1 runs it")
@pytest.mark.parametrize("k,n,res,L", [c for c in LARGE if c[:2] != DEFAULT])
def test_large_fermat_matches_golden_slow(lib, k, n, res, L):
    _check(lib, k, n, res, L)


def test_served_large_request_matches_golden(lib):
    """1021*2^2300003-1 arrives first; small Fermat and LLR requests arrive while it runs and
    share its batch.  The large verdict equals the golden residue."""
    from ahnum_gb300 import serve
    k, n, res, L = LARGE[0]
    small = serve.poisson_requests(seed=5, rate_per_s=4.0, duration_s=3.0, n_range=(20_000, 60_000))
    reqs = [serve.Request(0, serve.FERMAT, k, n, 0.0)]
    reqs += [serve.Request(i + 1, r.kind, r.k, r.n, r.arrival) for i, r in enumerate(small)]
    srv = serve.Server(gerbicz_block=1000)
    try:
        verdicts, stats = srv.serve(reqs)
    finally:
        srv.close()
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["peak_active"] >= 2
    big = next(v for v in verdicts if v.rid == 0)
    assert big.fft_len == L
    assert big.res64 == res, f"{big.res64:016X} != {res:016X}"
    assert not big.is_prime and big.maxerr < 0.4
