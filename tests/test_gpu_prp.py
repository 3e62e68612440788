"""End-to-end Fermat and LLR tests on the CUDA backend against the reference's golden residues.

Known residues: tests/known_residues.csv of the reference (GMP, primecrunch and known primes,
rows with n <= 100000 as its run_known.sh does, plus the config-size rows), the LLR results its
CMakeLists.txt:86-90 pins against PRST 14.0.1888, the Gerbicz fault test of CMakeLists.txt:95
and the LLR fault matrix of tests/test_llr.c.  The values are restated here as data.
"""
import os

import pytest

pytestmark = pytest.mark.gpu

# (k, n, RES64) -- reference tests/known_residues.csv rows with n <= 100000
KNOWN = [
    (9357, 20000, 0x79291CD2F47CE48C),
    (8191, 25000, 0xD45538E6F07266C6),
    (3, 26459, 0x1),
    (5, 30000, 0xB7980452FDBC4183),
    (7, 40001, 0xEB4ADF0EC94C09E6),
    (3, 41628, 0x1),
    (1, 44497, 0x1),
    (1365, 45678, 0xEF89209BAE5FF19A),
    (9999, 60000, 0x1C248905164FFD34),
    (4095, 70000, 0xEB8AD04F6137E373),
    (1203, 90001, 0x4BE9F1953E350085),
    (33, 99999, 0xE515A5DE4F8FEEC1),
]


@pytest.mark.parametrize("k,n,res", KNOWN)
def test_known_residue(lib, k, n, res):
    from ahnum_gb300.kite import prp
    r = prp(k, n)
    assert r.rc == 0
    assert r.res64 == res, f"{k}*2^{n}-1: {r.res64:016X} != {res:016X}"
    assert r.is_prp == (res == 1)
    assert r.maxerr < 0.4
    assert r.gerbicz_errors == 0


def test_gerbicz_fault_detected_and_rolled_back(lib):
    """reference CMakeLists.txt:95: a +1 on one digit at iteration 50000 is caught by the
    Gerbicz check, rolled back, and the residue is still right"""
    from ahnum_gb300.kite import prp
    r = prp(1203, 90001, inject_fault_at=50000)
    assert r.rc == 0
    assert r.res64 == 0x4BE9F1953E350085
    assert r.gerbicz_errors >= 1


def test_config_size_primecrunch_residue(lib):
    """9357*2^369717-1 at FFT length 28672 (the single-test size at ~13 bits/word),
    block 1000, against the primecrunch residue in known_residues.csv"""
    from ahnum_gb300.kite import prp
    r = prp(9357, 369717, fft_len=28672, gerbicz_block=1000)
    assert r.rc == 0 and r.fft_len == 28672
    assert r.res64 == 0xF5FDA01218F20439
    assert r.maxerr < 0.4


def test_config2_size_known_prime(lib):
    """9001*2^662695-1 (known prime) at FFT length 49152"""
    from ahnum_gb300.kite import prp
    r = prp(9001, 662695, fft_len=49152)
    assert r.rc == 0 and r.is_prp and r.res64 == 1
    assert r.maxerr < 0.4


def test_checkpoint_resume(lib, tmp_path):
    """a stopped test resumes from its verified checkpoint to the same residue"""
    import ctypes as C
    from ahnum_gb300 import native
    lib_ = native.load()
    path = str(tmp_path / "ck")
    flag = C.c_int(0)
    state = {"stop": True}

    def progress(arg, it, n, e):
        if state["stop"] and it >= 30000:
            flag.value = 1

    cb = native.PROGRESS_FN(progress)
    o = native.KitePrpOpts()
    o.fft = native.KiteOpts(native.KITE_BACKEND_CUDA, 0, 0, 0)
    o.checkpoint = path.encode()
    o.progress = cb
    o.abort_flag = C.pointer(flag)
    r = native.KitePrpResult()
    rc = lib_.kite_prp(9999, 60000, 3, C.byref(o), C.byref(r))
    assert rc == -5  # KITE_PRP_ABORTED
    it = C.c_uint64()
    assert lib_.kite_prp_checkpoint_iter(path.encode(), 9999, 60000, 3, C.byref(it)) == 0
    assert it.value > 0
    flag.value = 0
    state["stop"] = False
    r2 = native.KitePrpResult()
    rc = lib_.kite_prp(9999, 60000, 3, C.byref(o), C.byref(r2))
    assert rc == 0 and r2.resumed and r2.resumed_at == it.value
    assert r2.res64 == 0x1C248905164FFD34


LLR = [
    (3, 26459, None),
    (3, 41628, None),
    (9357, 20000, 0xDC52061161A0DE1C),
    (9357, 25000, 0x54A27E03D75F2447),
    (33, 99999, 0x3FAF838186E8A836),
]


@pytest.mark.parametrize("k,n,res", LLR)
def test_llr_known(lib, k, n, res):
    from ahnum_gb300.kite import llr
    r = llr(k, n)
    assert r.rc == 0
    if res is None:
        assert r.is_prime
    else:
        assert not r.is_prime and r.res64 == res
        assert r.confirm_runs == 1  # confirmed by a second run at a longer FFT


def test_llr_fault_in_run0_of_prime_outvoted(lib):
    """reference tests/test_llr.c:69-74"""
    from ahnum_gb300.kite import llr
    r = llr(3, 41628, inject_fault_at=20000)
    assert r.rc == 0 and r.is_prime and r.confirm_runs == 2


def test_llr_fault_in_run0_of_composite(lib):
    """reference tests/test_llr.c:76-80"""
    from ahnum_gb300.kite import llr
    r = llr(9357, 25000, inject_fault_at=12000)
    assert r.rc == 0 and not r.is_prime and r.res64 == 0x54A27E03D75F2447


def test_llr_roundoff_fault_retries_longer_fft(lib):
    from ahnum_gb300.kite import llr
    r = llr(9357, 25000, inject_roundoff_at=5000)
    assert r.rc == 0 and r.res64 == 0x54A27E03D75F2447 and r.roundoff_retries >= 1
    r = llr(9357, 25000, inject_roundoff_ladder=1)
    assert r.rc == 0 and r.res64 == 0x54A27E03D75F2447 and r.roundoff_retries >= 1
