"""kc_square_noalloc: the squaring for callers that cannot allocate device memory when they
need it (a plugin inside a host that owns the device memory through its own pool, or a loop
that cannot take an allocation's synchronisation).  Its scratch lives in a static device array,
so these checks compare it, call after call, with the ordinary kc_square, which uses the
scratch its engine allocated; the results must be bit-identical.

This file is collected last: it runs after every other test, and it also passes alone in a
fresh process."""
import ctypes as C
import random

import pytest

pytestmark = pytest.mark.gpu

# include/kite_cuda.h: below -10000, apart from negated CUDA error codes
KC_NOALLOC_TOO_LARGE = -10001
KC_NOALLOC_BAD_ARGUMENT = -10002


def _engine(lib, k, n, L):
    e = lib.kc_engine_new(k, n, L, None, None, None, 0, 0, 0, 0, -1)
    assert e, (k, n, L)
    return e


def _digits(lib, e, x, L):
    d = (C.c_int64 * L)()
    assert lib.kc_to_digits(e, x, d) == 0
    return bytes(d)


def _seeded_number(lib, e, k, n, L, seed):
    nl = (n + 127) // 64
    N = k * (1 << n) - 1
    v = random.Random(seed).randrange(N)
    limbs = (C.c_uint64 * nl)(*[(v >> (64 * i)) & (2**64 - 1) for i in range(nl)])
    d = (C.c_int64 * L)()
    assert lib.kc_limbs_to_digits(k, n, L, limbs, d) == 0
    x = lib.kc_num_alloc(e)
    assert x and lib.kc_from_digits(e, x, d) == 0
    return x


@pytest.mark.parametrize("k,n,L", [(9357, 20000, 1344), (9001, 662695, 49152), (3, 900000, 65536)])
def test_noalloc_matches_kc_square_two_calls(lib, k, n, L):
    e = _engine(lib, k, n, L)
    try:
        a = _seeded_number(lib, e, k, n, L, seed=n)
        b = _seeded_number(lib, e, k, n, L, seed=n)
        out = lib.kc_num_alloc(e)
        assert out
        for call in range(2):
            assert lib.kc_square(e, a, 1) == 0
            src = b if call == 0 else out
            assert lib.kc_square_noalloc(e, src, out) == 0
            assert _digits(lib, e, out, L) == _digits(lib, e, a, L), f"call {call}"
        # in place, too
        assert lib.kc_square(e, a, 1) == 0
        assert lib.kc_square_noalloc(e, out, out) == 0
        assert _digits(lib, e, out, L) == _digits(lib, e, a, L)
        assert lib.kc_error(e) == 0
        assert 0 < lib.kc_maxerr(e) < 0.4
        for p in (a, b, out):
            lib.kc_num_free(e, p)
    finally:
        lib.kc_engine_free(e)


def test_noalloc_refuses_lengths_above_its_maximum(lib):
    e = _engine(lib, 3, 2000000, 131072)
    try:
        x = lib.kc_num_alloc(e)
        assert lib.kc_square_noalloc(e, x, x) == KC_NOALLOC_TOO_LARGE
        assert lib.kc_square_noalloc(e, None, x) == KC_NOALLOC_BAD_ARGUMENT
        assert lib.kc_error(e) == 0
        lib.kc_num_free(e, x)
    finally:
        lib.kc_engine_free(e)
