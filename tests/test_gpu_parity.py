"""GPU parity: modular arithmetic through the kite C API on the CUDA backend against exact
integer arithmetic and the CPU oracle.

The protocol follows the reference's randomized GMP comparison (tests/test_gmp.c:56-172):
round trip, 20 squarings, a product, a small multiple, add and sub each followed by a product,
a 30-step V^2-2 chain, and 3^(2^30); every result must be bit-exact.  Lengths are chosen to
cover every radix (2, 3, 4, 5, 7, 8) in both the row and the column transform, low bits per
word (k spanning several top digits), k = 1 (Mersenne, empty top region) and large k.
"""
import random

import pytest

pytestmark = pytest.mark.gpu

# (k, n, L); L = 0 lets the library choose as the reference does
CASES = [
    (9357, 20000, 0),
    (1, 44497, 0),
    (3, 26459, 0),
    (1365, 45678, 0),
    (9999, 60000, 0),
    (5, 30000, 2560),     # 2^9 * 5
    (7, 40001, 3584),     # 2^9 * 7
    (33, 25000, 2240),    # 2^6 * 5 * 7 : low bits/word
    (8191, 25000, 3456),  # 2^7 * 3^3
    (1203, 9001, 1600),   # 2^6 * 5^2, ~5.6 bits/word
    (4095, 70000, 6144),
]


@pytest.mark.parametrize("k,n,L", CASES)
def test_gmp_protocol(lib, k, n, L):
    from ahnum_gb300.kite import Ctx
    rng = random.Random(k * 1000003 + n)
    with Ctx(k, n, L) as c:
        N = c.N
        a, b = rng.randrange(N), rng.randrange(N)
        x, y = c.num(a), c.num(b)
        assert c.get(x) == a, "round trip"
        c.square(x, 20)
        t = pow(a, 1 << 20, N)
        assert c.get(x) == t, "20 squarings"
        c.mul(x, y)
        t = t * b % N
        assert c.get(x) == t, "mul"
        c.mul_small(x, 3)
        t = t * 3 % N
        assert c.get(x) == t, "mul_small"
        c.add(x, y)
        c.square(x)
        t = (t + b) * (t + b) % N
        assert c.get(x) == t, "add+square"
        c.sub(x, y)
        t = (t - b) % N
        assert c.get(x) == t, "sub"
        two = c.num(2)
        c.set(x, 4)
        t = 4
        for _ in range(30):
            c.square(x)
            c.sub(x, two)
            t = (t * t - 2) % N
        assert c.get(x) == t, "llr chain"
        c.set(x, 3)
        c.square(x, 30)
        assert c.get(x) == pow(3, 1 << 30, N), "small start"
        e = c.maxerr()
        assert 0 <= e < 0.4, e
        c.check()


@pytest.mark.parametrize("k,n,L", [(9357, 20000, 0), (33, 25000, 2240), (8191, 25000, 3456)])
def test_matches_oracle_chain(lib, oracle_mod, k, n, L):
    """Same seeded input, 200 squarings and a product: identical residues, and a round-off of
    the same size as the oracle's."""
    from ahnum_gb300.kite import Ctx
    rng = random.Random(n)
    with Ctx(k, n, L) as c, oracle_mod.OracleCtx(k, n, c.L) as o:
        a, b = rng.randrange(c.N), rng.randrange(c.N)
        x, y = c.num(a), c.num(b)
        ox, oy = o.num(a), o.num(b)
        c.square(x, 200)
        o.square(ox, 200)
        c.mul(x, y)
        o.mul(ox, oy)
        assert c.get(x) == o.get(ox)
        ge, oe = c.maxerr(), o.maxerr()
        assert ge < 0.4 and oe < 0.4
        assert ge < 4 * oe + 0.02, (ge, oe)
