"""The exact integer-NTT engine (include/kite_ntt.h, KITE_BACKEND_CUDA_NTT) on the GPU: raw
squarings, products and V^2 - 2 steps against Python integers, the GMP chain fixtures, the
reference's known Fermat and LLR residues through kite_prp / kite_llr, and a bit-for-bit
cross-check against the FP64 IBDWT engine on the same inputs."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _nlimbs(n):
    return (n + 127) // 64


def _seeded_residue(seed, k, n):
    N = k * (1 << n) - 1
    rng = np.random.Generator(np.random.PCG64(seed))
    words = rng.integers(0, 2**64, size=_nlimbs(n), dtype=np.uint64)
    return int.from_bytes(words.astype("<u8").tobytes(), "little") % N


class Engine:
    """kn_* through ctypes, values as Python integers."""

    def __init__(self, k, n):
        from ahnum_gb300 import native
        self.lib = native.load()
        self.k, self.n = k, n
        self.N = k * (1 << n) - 1
        self.h = self.lib.kn_engine_new(k, n, -1)
        assert self.h
        self.nl = self.lib.kn_limbs(self.h)
        self.nums = []

    def num(self, v=0):
        x = self.lib.kn_num_alloc(self.h)
        assert x
        self.nums.append(x)
        self.set(x, v)
        return x

    def set(self, x, v):
        arr = (C.c_uint64 * self.nl)()
        C.memmove(arr, v.to_bytes(8 * self.nl, "little"), 8 * self.nl)
        assert self.lib.kn_set_limbs(self.h, x, arr) == 0

    def get(self, x):
        arr = (C.c_uint64 * self.nl)()
        assert self.lib.kn_get_limbs(self.h, x, arr) == 0
        return int.from_bytes(C.string_at(arr, 8 * self.nl), "little")

    def close(self):
        for x in self.nums:
            self.lib.kn_num_free(self.h, x)
        self.lib.kn_engine_free(self.h)


SIZES = [(3, 64), (3, 1000), (9357, 20000), (1203, 90001), (187, 100003), (4733, 369717), (9999, 662695),
         ((1 << 30) - 1, 20011)]


@pytest.mark.parametrize("k,n", SIZES)
def test_squarings_products_and_steps_exact(lib, k, n):
    e = Engine(k, n)
    try:
        N = e.N
        assert 2 * e.lib.kn_num_words(e.h) <= e.lib.kn_transform_len(e.h)
        x0, y0 = _seeded_residue(7, k, n), _seeded_residue(8, k, n)
        x, y = e.num(x0), e.num(y0)
        assert e.get(x) == x0
        sq = 40 if n < 200000 else 12
        assert e.lib.kn_square(e.h, x, sq) == 0
        assert e.get(x) == pow(x0, 1 << sq, N)
        assert e.lib.kn_mul(e.h, x, y) == 0
        assert e.get(x) == pow(x0, 1 << sq, N) * y0 % N
        e.set(x, x0)
        assert e.lib.kn_square_add(e.h, x, 5, -2) == 0
        v = x0
        for _ in range(5):
            v = (v * v - 2) % N
        assert e.get(x) == v
        # edge values: 0, 1, N - 1
        for v in (0, 1, N - 1):
            e.set(x, v)
            e.lib.kn_square(e.h, x, 3)
            assert e.get(x) == pow(v, 8, N)
        assert e.lib.kn_error(e.h) == 0
    finally:
        e.close()


def _load(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


CHAINS = [c for c in _load("chains.json") if c["name"] in ("cpu_small", "cpu_mid", "single_28672")]


@pytest.mark.parametrize("c", CHAINS, ids=[c["name"] for c in CHAINS])
def test_chain_matches_gmp(lib, c):
    e = Engine(c["k"], c["n"])
    try:
        x = e.num(_seeded_residue(c["x0_seed"], c["k"], c["n"]))
        assert e.lib.kn_square(e.h, x, c["squarings"]) == 0
        v = e.get(x)
        assert hashlib.sha256(v.to_bytes(8 * _nlimbs(c["n"]), "little")).hexdigest() == c["sha256_limbs"]
    finally:
        e.close()


KNOWN = [(9357, 20000, 0x79291CD2F47CE48C), (3, 26459, 0x1), (1, 44497, 0x1), (9999, 60000, 0x1C248905164FFD34),
         (1203, 90001, 0x4BE9F1953E350085)]


@pytest.mark.parametrize("k,n,res", KNOWN)
def test_known_residue_through_kite_prp(lib, k, n, res):
    from ahnum_gb300.kite import CUDA_NTT, prp
    r = prp(k, n, backend=CUDA_NTT)
    assert r.rc == 0 and r.res64 == res and r.is_prp == (res == 1)
    assert r.maxerr == 0.0 and r.gerbicz_errors == 0


def test_gerbicz_fault_on_ntt(lib):
    from ahnum_gb300.kite import CUDA_NTT, prp
    r = prp(1203, 90001, inject_fault_at=50000, backend=CUDA_NTT)
    assert r.rc == 0 and r.res64 == 0x4BE9F1953E350085 and r.gerbicz_errors >= 1


@pytest.mark.parametrize("k,n,res", [(3, 41628, None), (9357, 25000, 0x54A27E03D75F2447)])
def test_llr_through_kite_llr(lib, k, n, res):
    from ahnum_gb300.kite import CUDA_NTT, llr
    r = llr(k, n, backend=CUDA_NTT)
    assert r.rc == 0
    if res is None:
        assert r.is_prime
    else:
        assert not r.is_prime and r.res64 == res


def test_config1_fermat_residue(lib):
    """the full seeded config-1 Fermat test (k = 4733, n = 369717) against GMP's residue"""
    from ahnum_gb300.kite import CUDA_NTT, prp
    want = [c for c in _load("fermat.json") if c["name"] == "config1_full"][0]
    r = prp(want["k"], want["n"], gerbicz_block=1000, backend=CUDA_NTT)
    assert r.rc == 0 and format(r.res64, "016X") == want["res64"]


def test_cross_check_with_fp64_engine(lib):
    """the same residue squared 3000 times by both engines: identical values"""
    from ahnum_gb300.kite import Ctx
    k, n = 9001, 662695
    x0 = _seeded_residue(99, k, n)
    with Ctx(k, n, 49152) as g:
        x = g.num(x0)
        g.square(x, 3000)
        v_fp = g.get(x)
        assert g.maxerr() < 0.4
    e = Engine(k, n)
    try:
        x = e.num(x0)
        e.lib.kn_square(e.h, x, 3000)
        assert e.get(x) == v_fp
    finally:
        e.close()


def test_group_squares_every_member(lib):
    """a group of tests with different k, n and transform lengths: graph chunks plus a remainder,
    every member exact"""
    from ahnum_gb300 import native
    sizes = [(3, 1000), (9357, 20000), (1203, 90001), (4733, 369717), (7, 7)]
    engines = [Engine(k, n) for k, n in sizes if n >= 8]
    g = lib.kn_group_new(-1)
    assert g
    try:
        xs, want = [], []
        for i, e in enumerate(engines):
            v = _seeded_residue(200 + i, e.k, e.n)
            x = e.num(v)
            xs.append(x)
            want.append(pow(v, 1 << 21, e.N))
            assert lib.kn_group_add(g, e.h, x) == i
        assert lib.kn_group_add(g, engines[0].h, xs[0]) == -1  # an engine joins once
        ms = C.c_float(0)
        assert lib.kn_group_square(g, 21, C.byref(ms)) == 0
        assert ms.value > 0
        for e, x, w in zip(engines, xs, want):
            assert e.get(x) == w
    finally:
        lib.kn_group_free(g)
        for e in engines:
            e.close()


def test_ntt_fermat_batch_known_residues(lib):
    """a lockstep Gerbicz batch on NTT groups: tests of different n leave the lockstep as they
    near their end and finish alone; every RES64 equals the reference's known residue, and a
    fault injected in one test is caught by its check and rolled back"""
    from ahnum_gb300.ntt_group import NttFermatBatch
    want = {(9357, 20000): 0x79291CD2F47CE48C, (3, 26459): 0x1, (1, 44497): 0x1,
            (9999, 60000): 0x1C248905164FFD34, (1203, 90001): 0x4BE9F1953E350085}
    with NttFermatBatch(list(want), block=1000, blocks_per_check=10) as b:
        b.fault = (9999, 13000)
        res = b.run()
        assert b.blocks > 0 and b.block_ms > 0
    for r in res:
        assert r["res64"] == want[(r["k"], r["n"])], (r["k"], r["n"], hex(r["res64"]))
        assert r["is_prp"] == (want[(r["k"], r["n"])] == 1)
        assert r["gerbicz_errors"] == (1 if r["k"] == 9999 else 0)


LARGE = _load("chains_large.json")


@pytest.mark.parametrize("c", LARGE, ids=[c["name"] for c in LARGE])
def test_large_chain_matches_gmp(lib, c):
    """the large single-test regime (n in [2e7, 2.5e7]): transform length 2^20, the 1024 x 1024
    four-step, against GMP's chain"""
    e = Engine(c["k"], c["n"])
    try:
        assert e.lib.kn_transform_len(e.h) == 1 << 20
        x = e.num(_seeded_residue(c["x0_seed"], c["k"], c["n"]))
        assert e.lib.kn_square(e.h, x, c["squarings"]) == 0
        v = e.get(x)
        assert hashlib.sha256(v.to_bytes(8 * _nlimbs(c["n"]), "little")).hexdigest() == c["sha256_limbs"]
    finally:
        e.close()
