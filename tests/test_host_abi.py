"""The C-ABI library on the CPU: it loads, exports every function include/*.h declares, and its
exact host layer (layout, weights, carry with fold, limbs) agrees with the oracle and with exact
integer arithmetic.  No GPU and no compute call on a device."""
import ctypes as C
import os
import random
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = []
    for h in ("kite.h", "kite_cuda.h", "kite_proof.h", "kite_ntt.h"):
        with open(os.path.join(ROOT, "include", h)) as f:
            src = f.read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b([a-z_][a-z0-9_]*)\s*\(", src):
            name = m.group(1)
            if name.startswith(("kite_", "kc_", "pp_", "kn_")) and not name.endswith("_fn"):
                names.append(name)
    # drop function-pointer field names inside structs
    return sorted(set(n for n in names if n not in ("progress", "on_point", "on_confirm")))


def test_library_exports_every_declared_function(lib):
    declared = _declared_functions()
    assert len(declared) > 40
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_declares_every_header_function(lib):
    from ahnum_gb300 import native
    assert set(_declared_functions()) <= set(native.PROTOTYPES)


@pytest.mark.parametrize("k,n,L", [(9357, 369717, 28672), (9001, 662695, 49152), (1, 44497, 2560),
                                   (255, 20000000, 1179648), (3, 1000, 64), (9999, 60000, 3584)])
def test_layout_identical_to_oracle(lib, oracle_mod, k, n, L):
    import numpy as np
    bits = (C.c_uint8 * L)()
    w = (C.c_double * L)()
    osc = (C.c_double * L)()
    meta = (C.c_uint64 * 5)()
    assert lib.kc_layout(k, n, L, bits, w, osc, meta) == 0
    with oracle_mod.OracleCtx(k, n, L) as o:
        ob, ow, oo, om = o.layout()
    assert bytes(bits) == ob
    assert np.array_equal(np.frombuffer(w, dtype=np.float64).view(np.uint64),
                          np.array(ow, dtype=np.float64).view(np.uint64))
    assert np.array_equal(np.frombuffer(osc, dtype=np.float64).view(np.uint64),
                          np.array(oo, dtype=np.float64).view(np.uint64))
    assert list(meta) == om


def _positions(k, n, L):
    bits = (C.c_uint8 * L)()
    from ahnum_gb300 import native
    native.load().kc_layout(k, n, L, bits, None, None, None)
    s = [0]
    for b in bits:
        s.append(s[-1] + b)
    return s


@pytest.mark.parametrize("k,n,L", [(9357, 20000, 1344), (1, 44497, 2560), (7, 5000, 512), (3, 1000, 64)])
def test_digits_limbs_round_trip_and_carry(lib, k, n, L):
    N = k * (1 << n) - 1
    nl = (n + 127) // 64
    s = _positions(k, n, L)
    rng = random.Random(L)
    for _ in range(5):
        v = rng.randrange(N)
        limbs = (C.c_uint64 * nl)(*[(v >> (64 * i)) & (2**64 - 1) for i in range(nl)])
        d = (C.c_int64 * L)()
        assert lib.kc_limbs_to_digits(k, n, L, limbs, d) == 0
        # stored form is v/k: k * sum(d_j 2^{s_j}) == v (mod N)
        assert (k * sum(int(d[j]) << s[j] for j in range(L)) - v) % N == 0
        out = (C.c_uint64 * nl)()
        assert lib.kc_digits_to_limbs(k, n, L, d, out) == 0
        assert sum(int(out[i]) << (64 * i) for i in range(nl)) == v
        # unbalanced digits (products before the carry) carry to the same value
        big = [rng.randrange(-2**50, 2**50) for _ in range(L)]
        d2 = (C.c_int64 * L)(*big)
        assert lib.kc_carry_digits(k, n, L, d2) == 0
        val = lambda dd: (k * sum(int(dd[j]) << s[j] for j in range(L))) % N
        assert val(d2) == val(big)
        for j in range(L - 1):
            if j < L - 4:
                b = s[j + 1] - s[j]
                assert -(1 << (b - 1)) <= d2[j] < (1 << (b - 1))


def test_choose_fft_len_matches_oracle(lib, oracle_mod):
    rng = random.Random(7)
    for _ in range(40):
        k = rng.randrange(1, 10000) | 1
        n = rng.randrange(300000, 700001)
        assert lib.kc_choose_fft_len(k, n) == oracle_mod.choose_fft_len(k, n)
    assert oracle_mod.choose_fft_len(9357, 369717) > 0


def test_ctx_new_rejects_cpu_backends(lib):
    """no CPU fallback: the reference's CPU backend ids are refused (returns NULL) without a GPU
    being touched"""
    from ahnum_gb300 import native
    for b in (1, 2, 3, 4):
        o = native.KiteOpts(b, 0, 0, 0)
        assert not lib.kite_ctx_new(9357, 20000, -1, C.byref(o))
    o = native.KiteOpts(5, 0, 0, 0)
    assert not lib.kite_ctx_new(9358, 20000, -1, C.byref(o))  # even k
    assert not lib.kite_ctx_new(9357, 20000, 1, C.byref(o))   # c != -1


def test_latency_shapes_validated_and_loaded(lib):
    """the single-test shape overrides refuse shapes the engine cannot run, and the shipped
    GB300 tuning files load without a GPU"""
    from ahnum_gb300.tune import LATENCY_FILE, THROUGHPUT_FILE
    assert lib.kc_set_latency_shape(49152, 96, 3) != 0      # G not in {2, 4, 8}
    assert lib.kc_set_latency_shape(49152, 100, 2) != 0     # R does not divide H
    assert lib.kc_set_latency_shape(49152, 2048, 2) != 0    # C = 12: below 16
    assert lib.kc_set_latency_shape(49152, 96, 2) == 0
    assert lib.kc_set_latency_shape(49152, 0, 0) == 0       # back to the model
    assert lib.kc_tuning_load(LATENCY_FILE.encode()) >= 2
    assert lib.kc_tuning_load(THROUGHPUT_FILE.encode()) >= 10
    # leave the process as it was: no shapes, no measured times (they steer the length choice)
    for path in (LATENCY_FILE, THROUGHPUT_FILE):
        with open(path) as f:
            for line in f:
                if not line.startswith("#") and line.split():
                    L = int(line.split()[0])
                    lib.kc_set_latency_shape(L, 0, 0)
                    lib.kc_set_fft_shape(L, 0)
                    lib.kc_set_fft_time(L, 0.0)


def test_length_chooser_respects_the_reference_model(lib):
    """Every length the chooser picks is a usable four-step length (a multiple of 64 with no
    prime factor above 7) and holds the test within the reference's bits-per-word model
    (src/ctx.c:26-33, 107-141), for a seeded spread of k and n."""
    import random
    from ahnum_gb300.tune import safe_bpw, usable_lengths
    rng = random.Random(11)
    usable = set(usable_lengths(1024, 4 << 20))
    for _ in range(200):
        k = rng.randrange(1, 10000) | 1
        n = int(10 ** rng.uniform(4.3, 7.3))
        L = lib.kc_choose_fft_len(k, n)
        assert L in usable, (k, n, L)
        assert n / L <= safe_bpw(L, k) + 1e-9, (k, n, L)


def test_usable_lengths_are_seven_smooth_multiples_of_64():
    from ahnum_gb300.tune import usable_lengths
    got = usable_lengths(16384, 20480)
    # 2^14, 2^7 3^3 5, 2^9 5 7, 2^11 3^2, 2^7 3 7^2, 2^8 3 5^2, 2^6 3^2 5 7, 2^12 5
    assert got == [16384, 17280, 17920, 18432, 18816, 19200, 20160, 20480]
    for L in usable_lengths(1 << 16, 1 << 18):
        x = L
        for p in (2, 3, 5, 7):
            while x % p == 0:
                x //= p
        assert x == 1 and L % 64 == 0


def test_llr_choose_P_matches_oracle(lib, oracle_mod):
    """P = the smallest P >= 1 with Jacobi(P^2+4 | N) != 1, and the factor of 4P(P^2+4) and N,
    from the library's word-size symbol (N mod 4a) against the oracle's restatement of the
    reference (src/llr.c:33-93), over seeded k, n including small and huge n"""
    import ctypes as C
    import random
    rng = random.Random(77)
    lo = oracle_mod.load()
    factors = 0
    for _ in range(400):
        k = rng.randrange(1, 1 << 20) | 1
        n = rng.choice([rng.randrange(3, 200), rng.randrange(200, 10**6), rng.randrange(10**6, 10**8)])
        P1, f1 = C.c_uint32(), C.c_uint64()
        P2, f2 = C.c_uint32(), C.c_uint64()
        assert lib.kite_llr_choose_P(k, n, C.byref(P1), C.byref(f1)) == lo.ko_llr_choose_P(k, n, C.byref(P2), C.byref(f2))
        assert (P1.value, f1.value) == (P2.value, f2.value), (k, n)
        factors += f1.value != 0
    assert factors > 0
