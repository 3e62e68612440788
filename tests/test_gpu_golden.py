"""GPU results against the GMP fixtures in tests/golden (generated by make_golden.py) at the
benchmark sizes: the 10^4-squaring chain at n = 369717 and FFT length 28672, a chain at
FFT length 49152, the large single-test regime (n in [2e7, 2.5e7], FFT ~1.6-1.8 M words), and
full seeded Fermat residues.  Every comparison is exact: SHA-256 of the canonical limbs, RES64.
The large regime also checks a Gerbicz fault: a digit error injected part-way is detected,
rolled back, and the verified state equals a run without the fault."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _load(name):
    p = os.path.join(GOLDEN, name)
    if not os.path.exists(p):
        return []
    with open(p) as f:
        return json.load(f)


def _nlimbs(n):
    return (n + 127) // 64


def _seeded_residue(seed, k, n):
    N = k * (1 << n) - 1
    rng = np.random.Generator(np.random.PCG64(seed))
    words = rng.integers(0, 2**64, size=_nlimbs(n), dtype=np.uint64)
    return int.from_bytes(words.astype("<u8").tobytes(), "little") % N


def _sha(v, n):
    return hashlib.sha256(v.to_bytes(8 * _nlimbs(n), "little")).hexdigest()


LENGTH = {"single_28672": 28672, "single_49152": 49152}
CHAINS = [c for c in _load("chains.json") if c["name"] in ("single_28672", "single_49152", "mersenne_44497")]


@pytest.mark.parametrize("c", CHAINS, ids=[c["name"] for c in CHAINS])
def test_chain_matches_gmp(lib, c):
    from ahnum_gb300.kite import Ctx
    with Ctx(c["k"], c["n"], LENGTH.get(c["name"], 0)) as g:
        x = g.num(_seeded_residue(c["x0_seed"], c["k"], c["n"]))
        g.square(x, c["squarings"])
        v = g.get(x)
        assert _sha(v, c["n"]) == c["sha256_limbs"]
        assert format(v & (2**64 - 1), "016X") == c["low64"]
        assert g.maxerr() < 0.4


LARGE = _load("chains_large.json")


@pytest.mark.parametrize("c", LARGE, ids=[c["name"] for c in LARGE])
def test_large_chain_matches_gmp(lib, c):
    from ahnum_gb300.kite import Ctx
    with Ctx(c["k"], c["n"]) as g:
        assert 1_100_000 < g.L < 1_800_000
        x = g.num(_seeded_residue(c["x0_seed"], c["k"], c["n"]))
        g.square(x, c["squarings"])
        assert _sha(g.get(x), c["n"]) == c["sha256_limbs"]
        assert g.maxerr() < 0.4


def _latency_lines():
    from ahnum_gb300.tune import LATENCY_FILE
    with open(LATENCY_FILE) as f:
        return [tuple(int(float(v)) for v in line.split()) for line in f
                if not line.startswith("#") and len(line.split()) == 5]


TUNED = {c["name"]: c for c in LARGE + CHAINS if c["name"] in ("large_a", "single_49152")}


@pytest.mark.parametrize("name", sorted(TUNED))
def test_shipped_latency_shapes_match_gmp(lib, name):
    """the single-test shapes shipped in the GB300 tuning file: the engine takes them, and the
    chain equals GMP's bit for bit"""
    from ahnum_gb300.kite import Ctx
    c = TUNED[name]
    L = LENGTH.get(name, 0) or lib.kc_choose_fft_len(c["k"], c["n"])
    line = next(t for t in _latency_lines() if t[0] == L)
    _, _, R, Cc, G = line
    assert lib.kc_set_latency_shape(L, R, G) == 0
    try:
        e = lib.kc_engine_new(c["k"], c["n"], L, None, None, None, 0, 0, 0, 0, -1)
        assert e
        r, cc = C.c_uint32(), C.c_uint32()
        lib.kc_shape(e, C.byref(r), C.byref(cc))
        assert (r.value, cc.value, lib.kc_group_width(e)) == (R, Cc, G)
        lib.kc_engine_free(e)
        with Ctx(c["k"], c["n"], L) as g:
            x = g.num(_seeded_residue(c["x0_seed"], c["k"], c["n"]))
            g.square(x, c["squarings"])
            assert _sha(g.get(x), c["n"]) == c["sha256_limbs"]
            assert g.maxerr() < 0.4
    finally:
        lib.kc_set_latency_shape(L, 0, 0)


FERMAT = _load("fermat.json")


@pytest.mark.parametrize("c", FERMAT, ids=[c["name"] for c in FERMAT])
def test_full_fermat_matches_gmp(lib, c):
    from ahnum_gb300.kite import prp
    L = 28672 if c["n"] == 369717 else 49152
    r = prp(c["k"], c["n"], fft_len=L, gerbicz_block=1000 if c["n"] == 369717 else 0)
    assert r.rc == 0 and r.fft_len == L
    assert format(r.res64, "016X") == c["res64"]
    assert r.is_prp == c["is_prp"]
    assert r.maxerr < 0.4


def _segment(k, n, stop_at, fault_at, path):
    """kite_prp on the CUDA backend, stopped once `stop_at` squarings are verified; returns the
    result and the verified checkpoint's x and d limbs."""
    from ahnum_gb300 import native
    lib = native.load()
    flag = C.c_int(0)

    def progress(arg, it, nn, e):
        if it >= stop_at:
            flag.value = 1

    cb = native.PROGRESS_FN(progress)
    o = native.KitePrpOpts()
    o.fft = native.KiteOpts(native.KITE_BACKEND_CUDA, 0, 0, 0)
    o.gerbicz_block = 1000
    o.gerbicz_blocks = 5
    o.checkpoint = path.encode()
    o.progress = cb
    o.abort_flag = C.pointer(flag)
    o.inject_fault_at = fault_at
    r = native.KitePrpResult()
    rc = lib.kite_prp(k, n, 3, C.byref(o), C.byref(r))
    with open(path, "rb") as f:
        raw = f.read()
    hdr = np.frombuffer(raw[:56], dtype="<u8")
    nl = int(hdr[5])
    limbs = np.frombuffer(raw[56:56 + 16 * nl], dtype="<u8")
    return rc, r, int(hdr[4]), limbs[:nl].tobytes(), limbs[nl:].tobytes()


def test_large_gerbicz_fault_rolled_back(lib, tmp_path):
    """the large single-test regime: a +1 on one digit after squaring 2500 is caught by the next
    Gerbicz check and rolled back; the verified state at 10000 squarings equals a fault-free
    run's, bit for bit"""
    k, n = 187, 24715281
    rc1, r1, it1, x1, d1 = _segment(k, n, 10000, 2500, str(tmp_path / "a"))
    rc2, r2, it2, x2, d2 = _segment(k, n, 10000, 0, str(tmp_path / "b"))
    assert rc1 == rc2 == -5  # stopped on request (KITE_PRP_ABORTED) after the check
    assert r1.gerbicz_errors >= 1 and r2.gerbicz_errors == 0
    assert it1 == it2 and it1 >= 10000
    assert x1 == x2 and d1 == d2
    assert r1.maxerr < 0.4 and r2.maxerr < 0.4
