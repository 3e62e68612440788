"""The Gerbicz check's comparison on the device (kc_equal, and the batch's per-slot verdicts):
a == b (mod N) decided from the two numbers' digits by an exact carry with the top fold, where
the reference converts both numbers to canonical limbs on the host (src/prp.c:291-296, :470-474).
Checked against Python integers on values whose digit vectors differ though the values agree,
and through the batch's Gerbicz check with an injected digit fault."""
import ctypes as C
import random

import pytest

pytestmark = pytest.mark.gpu


def _engine(lib, k, n, L=0):
    L = L or lib.kc_choose_fft_len(k, n)
    e = lib.kc_engine_new(k, n, L, None, None, None, 0, 0, 0, 0, -1)
    assert e
    return e, L


def _from_int(lib, e, k, n, L, v):
    nl = (n + 127) // 64
    limbs = (C.c_uint64 * nl).from_buffer_copy(v.to_bytes(8 * nl, "little"))
    d = (C.c_int64 * L)()
    assert lib.kc_limbs_to_digits(k, n, L, limbs, d) == 0
    x = lib.kc_num_alloc(e)
    assert lib.kc_from_digits(e, x, d) == 0
    return x, list(d)


def _from_digits(lib, e, digits):
    x = lib.kc_num_alloc(e)
    arr = (C.c_int64 * len(digits))(*digits)
    assert lib.kc_from_digits(e, x, arr) == 0
    return x


def _bits(lib, k, n, L):
    b = (C.c_uint8 * L)()
    w = (C.c_double * L)()
    o = (C.c_double * L)()
    m = (C.c_uint64 * 5)()
    assert lib.kc_layout(k, n, L, b, w, o, m) == 0
    return list(b)


@pytest.mark.parametrize("k,n,L", [(9357, 20000, 1344), (1, 44497, 0), (3, 100000, 0), (9001, 662695, 49152),
                                   (187, 24715281, 0)])
def test_equal_against_integers(lib, k, n, L):
    e, L = _engine(lib, k, n, L)
    rng = random.Random(n)
    N = k * (1 << n) - 1
    bits = _bits(lib, k, n, L)
    nums = []
    try:
        v = rng.randrange(N)
        x, dx = _from_int(lib, e, k, n, L, v)
        nums.append(x)
        # the same value in other digit vectors: carries moved between neighbouring digits
        moved = list(dx)
        for _ in range(50):
            j = rng.randrange(L - 1)
            c = rng.randrange(-2, 3)
            moved[j] += c << bits[j]
            moved[j + 1] -= c
        y = _from_digits(lib, e, moved)
        nums.append(y)
        assert lib.kc_equal(e, x, y) == 1
        # a value one apart, and one at random
        z, _ = _from_int(lib, e, k, n, L, (v + 1) % N)
        w, _ = _from_int(lib, e, k, n, L, rng.randrange(N))
        nums += [z, w]
        assert lib.kc_equal(e, x, z) == 0
        assert lib.kc_equal(e, z, x) == 0
        assert lib.kc_equal(e, x, w) == 0
        # products that agree as residues: (v^2)^2 from two squarings, against v^4 set from
        # limbs (Python integers, up to a million bits) and against two multiplications (the
        # product kernels, which leave other digit vectors)
        sq = lib.kc_num_alloc(e)
        nums.append(sq)
        assert lib.kc_copy(e, sq, x) == 0
        assert lib.kc_square(e, sq, 2) == 0
        if n <= 1_000_000:
            p4, _ = _from_int(lib, e, k, n, L, pow(v, 4, N))
            nums.append(p4)
            assert lib.kc_equal(e, sq, p4) == 1
            assert lib.kc_equal(e, p4, sq) == 1
        m4, y = lib.kc_num_alloc(e), lib.kc_num_alloc(e)
        nums += [m4, y]
        assert lib.kc_copy(e, m4, x) == 0 and lib.kc_copy(e, y, x) == 0
        assert lib.kc_mul(e, m4, y) == 0 and lib.kc_copy(e, y, m4) == 0 and lib.kc_mul(e, m4, y) == 0
        assert lib.kc_equal(e, sq, m4) == 1
        # digits hold the stored value x/k: the digit vector of -1 is x = -k (mod N)
        mk, _ = _from_int(lib, e, k, n, L, N - k)
        neg = _from_digits(lib, e, [-1] + [0] * (L - 1))
        zero = _from_digits(lib, e, [0] * L)
        nums += [mk, neg, zero]
        assert lib.kc_equal(e, mk, neg) == 1
        assert lib.kc_equal(e, neg, zero) == 0
        assert lib.kc_error(e) == 0
    finally:
        for p in nums:
            lib.kc_num_free(e, p)
        lib.kc_engine_free(e)


def test_batch_check_on_device_catches_a_fault(lib):
    """a +1 on one digit of x is caught by the next check (decided on the device), rolled back,
    and the test still ends at the golden residue; the check moves a few bytes per slot"""
    from ahnum_gb300.kite import Batch
    with Batch(gerbicz_block=200, gerbicz_blocks=4) as b:
        bad = b.add_fermat(9999, 60000)
        good = b.add_fermat(1365, 45678)
        b.step(2)
        assert lib.kc_batch_debug_corrupt(b.h, bad) == 0
        b.step(3)  # two more blocks, then the check block
        h2d, d2h = C.c_uint64(), C.c_uint64()
        lib.kc_batch_last_transfer(b.h, C.byref(h2d), C.byref(d2h))
        assert d2h.value < 64 * 8  # round-off words and the verdict words
        b.run()
        st, r = b.result(bad)
        assert st == 1 and r.rc == 0
        assert r.gerbicz_errors >= 1
        assert r.res64 == 0x1C248905164FFD34  # reference tests/known_residues.csv:10
        st, r2 = b.result(good)
        assert st == 1 and r2.res64 == 0xEF89209BAE5FF19A and r2.gerbicz_errors == 0
