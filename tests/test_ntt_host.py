"""Host-side parts of the integer-NTT engine (include/kite_ntt.h), without a GPU: the sizes it
picks for N = k*2^n - 1 (every convolution coefficient below the four primes' product, a transform
long enough for the acyclic product) and the exact conversions between canonical values and its
Montgomery-form words (x~ = x*2^n mod N)."""
import ctypes as C
import random

import pytest

PRIMES = (1053818881, 975175681, 943718401, 880803841)
PRODUCT = PRIMES[0] * PRIMES[1] * PRIMES[2] * PRIMES[3]

SIZES = [(3, 8), (3, 64), (1, 44497), (9357, 20000), (1203, 90001), (4733, 369717), (9999, 662695),
         ((1 << 30) - 1, 20011), (187, 24715281)]


def _layout(lib, k, n):
    w, W, NP = C.c_uint32(), C.c_uint32(), C.c_uint32()
    assert lib.kn_layout(k, n, C.byref(w), C.byref(W), C.byref(NP)) == 0
    return w.value, W.value, NP.value


@pytest.mark.parametrize("k,n", SIZES)
def test_sizes_bound_the_coefficients(lib, k, n):
    w, W, NP = _layout(lib, k, n)
    assert 24 <= w <= 50
    assert W * w >= n + 2 * k.bit_length() + 8       # room for values below (k + 1) 2^n, squared
    assert NP >= 2 * W and NP & (NP - 1) == 0 and NP <= 1 << 20
    assert W * ((1 << w) - 1) ** 2 < PRODUCT       # the CRT recovers every coefficient
    # no shorter power-of-2 transform exists for any admissible word size
    for ww in range(24, 51):
        WW = -(-(n + 2 * k.bit_length() + 8) // ww)
        if 2 * ww + (WW - 1).bit_length() + 1 <= 119:
            assert NP <= max(64, 1 << (2 * WW - 1).bit_length())


def test_out_of_range_refused(lib):
    w = C.c_uint32()
    assert lib.kn_layout(4, 1000, C.byref(w), None, None) != 0      # k even
    assert lib.kn_layout(1 << 30, 1000, None, None, None) != 0      # k too large
    assert lib.kn_layout(3, 7, None, None, None) != 0               # n too small


@pytest.mark.parametrize("k,n", SIZES[:7])
def test_montgomery_words_round_trip(lib, k, n):
    w, W, NP = _layout(lib, k, n)
    N = k * (1 << n) - 1
    nl = (n + 127) // 64
    rng = random.Random(k * 7919 + n)
    for v in (0, 1, 2, N - 1, rng.randrange(N), rng.randrange(N)):
        limbs = (C.c_uint64 * nl)()
        C.memmove(limbs, v.to_bytes(8 * nl, "little"), 8 * nl)
        words = (C.c_uint64 * W)()
        assert lib.kn_limbs_to_words(k, n, limbs, words) == 0
        assert all(words[j] < (1 << w) for j in range(W))
        mont = sum(words[j] << (w * j) for j in range(W))
        assert mont % N == v * pow(2, n, N) % N          # x~ = x 2^n mod N
        assert mont < (k + 1) << n                        # q + r 2^n with q < N / k, r < k
        back = (C.c_uint64 * nl)()
        assert lib.kn_words_to_limbs(k, n, words, back) == 0
        assert int.from_bytes(C.string_at(back, 8 * nl), "little") == v


def test_words_to_limbs_reduces_any_representative(lib):
    """the engine's results are Montgomery representatives below about (k + 1) 2^n: the
    conversion back reduces them fully"""
    k, n = 9357, 20000
    w, W, NP = _layout(lib, k, n)
    N = k * (1 << n) - 1
    nl = (n + 127) // 64
    rng = random.Random(5)
    for _ in range(4):
        mont = rng.randrange((k + 1) << n)
        words = (C.c_uint64 * W)(*[(mont >> (w * j)) & ((1 << w) - 1) for j in range(W)])
        back = (C.c_uint64 * nl)()
        assert lib.kn_words_to_limbs(k, n, words, back) == 0
        assert int.from_bytes(C.string_at(back, 8 * nl), "little") == mont * k % N
