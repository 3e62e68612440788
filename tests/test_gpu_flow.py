"""The persistent squaring kernel of the batched engine: its waits between CTAs are bounded.

A CTA of k_squarings that takes a work item first waits for the same test's previous phase.
If that work never comes, the wait gives up after its limit, raises the launch's timeout word,
and the launch ends; the host reads the word and reports an error instead of hanging.  This test
makes every wait run out on purpose (column items queued without their row items), with a short
limit, through the C ABI, and then checks that the GPU context still computes correctly."""
import ctypes as C
import random
import time

import pytest

pytestmark = pytest.mark.gpu


def _to_digits(lib, k, n, L, v):
    nl = (n + 127) // 64
    limbs = (C.c_uint64 * nl)(*[(v >> (64 * i)) & (2**64 - 1) for i in range(nl)])
    d = (C.c_int64 * L)()
    assert lib.kc_limbs_to_digits(k, n, L, limbs, d) == 0
    return d


def _from_digits(lib, k, n, L, d):
    nl = (n + 127) // 64
    limbs = (C.c_uint64 * nl)()
    assert lib.kc_digits_to_limbs(k, n, L, d, limbs) == 0
    return sum(int(limbs[i]) << (64 * i) for i in range(nl))


def test_persistent_kernel_waits_give_up_and_report(lib):
    k, n, L = 9357, 20000, 1344
    e = lib.kc_engine_new(k, n, L, None, None, None, 0, 0, 0, 0, -1)
    assert e
    try:
        t0 = time.perf_counter()
        # 10^8 SM cycles: about 50 ms at the GB300's clocks
        assert lib.kc_engine_wait_selftest(e, 100_000_000) == 1
        assert time.perf_counter() - t0 < 10
        assert lib.kc_error(e) == 0
        # the context still works: 5 squarings of a seeded residue equal exact arithmetic
        N = k * (1 << n) - 1
        a = random.Random(n).randrange(N)
        x = lib.kc_num_alloc(e)
        assert x and lib.kc_from_digits(e, x, _to_digits(lib, k, n, L, a)) == 0
        assert lib.kc_square(e, x, 5) == 0
        d = (C.c_int64 * L)()
        assert lib.kc_to_digits(e, x, d) == 0
        assert _from_digits(lib, k, n, L, d) % N == pow(a, 2 ** 5, N)
        assert lib.kc_error(e) == 0 and lib.kc_maxerr(e) < 0.4
        lib.kc_num_free(e, x)
    finally:
        lib.kc_engine_free(e)
