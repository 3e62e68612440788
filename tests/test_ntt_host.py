"""Host-side parts of the integer-NTT engine (include/kite_ntt.h), without a GPU: the sizes it
picks for N = k*2^n - 1 (every convolution coefficient below the four primes' product, a transform
long enough for the acyclic product) and the exact conversions between canonical values and its
Montgomery-form words (x~ = x*2^n mod N)."""
import ctypes as C
import random

import pytest

PRIMES = (1053818881, 975175681, 943718401, 880803841)


def _product(q):
    out = 1
    for p in PRIMES[:q]:
        out *= p
    return out

SIZES = [(3, 8), (3, 64), (1, 44497), (9357, 20000), (1203, 90001), (4733, 369717), (9999, 662695),
         ((1 << 30) - 1, 20011), (187, 24715281)]


def _layout(lib, k, n):
    q, w, W, NP = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint32()
    assert lib.kn_layout(k, n, C.byref(q), C.byref(w), C.byref(W), C.byref(NP)) == 0
    return q.value, w.value, W.value, NP.value


@pytest.mark.parametrize("k,n", SIZES)
def test_sizes_bound_the_coefficients(lib, k, n):
    q, w, W, NP = _layout(lib, k, n)
    assert q in (3, 4) and 24 <= w <= 50
    assert W * w >= n + 2 * k.bit_length() + 8       # room for values below (k + 1) 2^n, squared
    assert NP >= 2 * W and NP & (NP - 1) == 0 and NP <= 1 << 20
    assert W * ((1 << w) - 1) ** 2 < _product(q)   # the CRT recovers every coefficient
    # no choice of primes and admissible word size needs fewer prime-points
    for qq in (3, 4):
        for ww in range(24, 51):
            WW = -(-(n + 2 * k.bit_length() + 8) // ww)
            if WW * ((1 << ww) - 1) ** 2 < _product(qq):
                assert q * NP <= qq * max(64, 1 << (2 * WW - 1).bit_length())


def test_three_primes_where_they_save_work(lib):
    """n near 5e5: four primes need a 2^15 transform (w = 50), three primes (w <= 36) too, so
    three are chosen; near 3.5e5 four primes fit 2^14 and are kept"""
    assert _layout(lib, 4733, 500001)[0] == 3
    assert _layout(lib, 4733, 369717)[0] == 4


def test_out_of_range_refused(lib):
    w = C.c_uint32()
    assert lib.kn_layout(4, 1000, None, C.byref(w), None, None) != 0      # k even
    assert lib.kn_layout(1 << 30, 1000, None, None, None, None) != 0      # k too large
    assert lib.kn_layout(3, 7, None, None, None, None) != 0               # n too small


@pytest.mark.parametrize("k,n", SIZES[:7])
def test_montgomery_words_round_trip(lib, k, n):
    q, w, W, NP = _layout(lib, k, n)
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
    q, w, W, NP = _layout(lib, k, n)
    N = k * (1 << n) - 1
    nl = (n + 127) // 64
    rng = random.Random(5)
    for _ in range(4):
        mont = rng.randrange((k + 1) << n)
        words = (C.c_uint64 * W)(*[(mont >> (w * j)) & ((1 << w) - 1) for j in range(W)])
        back = (C.c_uint64 * nl)()
        assert lib.kn_words_to_limbs(k, n, words, back) == 0
        assert int.from_bytes(C.string_at(back, 8 * nl), "little") == mont * k % N


def test_split_members_balances_work_and_keeps_everyone():
    """NTT groups squared together are dealt members of about equal work (largest first, each
    to the lightest group); every member lands in exactly one group."""
    from ahnum_gb300.ntt_group import split_members
    sizes = [700000, 650000, 300000, 310000, 500000, 480000, 420000]
    parts = split_members(list(enumerate(sizes)), 2, size=lambda m: m[1])
    assert len(parts) == 2
    got = sorted(i for p in parts for i, _ in p)
    assert got == list(range(len(sizes)))
    loads = [sum(v for _, v in p) for p in parts]
    assert abs(loads[0] - loads[1]) <= max(sizes)
    # more parts than members: one member per part, none empty
    assert [len(p) for p in split_members([1, 2], 4)] == [1, 1]
    assert split_members([], 3) == [[]]


def test_residue_nm1_matches_oracle_with_shared_factors(oracle_mod):
    """base^(N+1) -> base^(N-1) in the NTT batch's Python finish, against the oracle's restatement
    of the reference's kite_residue_nm1, including N divisible by primes of the base"""
    import ctypes as C
    import random
    from ahnum_gb300.ntt_group import residue_nm1
    lib = oracle_mod.load()
    rng = random.Random(5)
    shared = 0
    for _ in range(150):
        k = rng.randrange(1, 3000) | 1
        n = rng.randrange(60, 400)
        N = k * (1 << n) - 1
        for base in (3, 5, 6, 15):
            y = rng.randrange(N)
            nl = (n + 127) // 64
            arr = (C.c_uint64 * nl)(*[(y >> (64 * i)) & (2**64 - 1) for i in range(nl)])
            Narr = (C.c_uint64 * nl)(*[(N >> (64 * i)) & (2**64 - 1) for i in range(nl)])
            rc = lib.ko_residue_nm1(arr, Narr, nl, base)
            want = sum(int(arr[i]) << (64 * i) for i in range(nl))
            assert rc == 0
            assert residue_nm1(y, N, base) == want, (k, n, base)
            shared += N % 3 == 0 or N % 5 == 0
    assert shared > 0
