"""Generates the golden fixtures in this directory with GMP (libgmp.so.10 through ctypes).

Inputs are seeded (numpy PCG64, one seed per workload), as the benchmark's synthetic workloads
are; the reference publishes no suite.  Outputs:

  chains.json    raw squaring chains: x0 uniform in [0, N) from seeded 64-bit limbs, squared
                 `count` times mod N; the SHA-256 of the result's little-endian limbs (the
                 kite_limbs(ctx) words) and its low word.  Includes the 10^4-squaring chain at
                 n = 369717 and smaller chains for the CPU suite.
  fermat.json    RES64 (low 64 bits of 3^(N-1) mod N) of seeded full Fermat tests at the
                 single-test sizes n = 369717 and n = 662695, and of a seeded mixed batch.

  chains_large.json  100-squaring chains at the large single-test size (n in [2e7, 2.5e7],
                 k odd in [3, 255]).

Usage:  python tests/golden/make_golden.py [chains|large|fermat|all]
The full Fermat residues take minutes each (GMP mpz_powm, one process per test).
"""
from __future__ import annotations

import ctypes as C
import ctypes.util
import hashlib
import json
import os
import sys
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class _Mpz(C.Structure):
    _fields_ = [("alloc", C.c_int), ("size", C.c_int), ("d", C.c_void_p)]


def _gmp():
    name = ctypes.util.find_library("gmp") or "libgmp.so.10"
    g = C.CDLL(name)
    g.__gmpz_init.argtypes = [C.POINTER(_Mpz)]
    g.__gmpz_clear.argtypes = [C.POINTER(_Mpz)]
    g.__gmpz_set_str.argtypes = [C.POINTER(_Mpz), C.c_char_p, C.c_int]
    g.__gmpz_get_str.argtypes = [C.c_char_p, C.c_int, C.POINTER(_Mpz)]
    g.__gmpz_get_str.restype = C.c_void_p
    g.__gmpz_powm.argtypes = [C.POINTER(_Mpz)] * 4
    g.__gmpz_sizeinbase.argtypes = [C.POINTER(_Mpz), C.c_int]
    g.__gmpz_sizeinbase.restype = C.c_size_t
    return g


def gmp_powm(base: int, exp: int, mod: int) -> int:
    g = _gmp()
    r, b, e, m = _Mpz(), _Mpz(), _Mpz(), _Mpz()
    for z in (r, b, e, m):
        g.__gmpz_init(C.byref(z))
    g.__gmpz_set_str(C.byref(b), format(base, "x").encode(), 16)
    g.__gmpz_set_str(C.byref(e), format(exp, "x").encode(), 16)
    g.__gmpz_set_str(C.byref(m), format(mod, "x").encode(), 16)
    g.__gmpz_powm(C.byref(r), C.byref(b), C.byref(e), C.byref(m))
    size = g.__gmpz_sizeinbase(C.byref(r), 16) + 2
    buf = C.create_string_buffer(size)
    g.__gmpz_get_str(buf, 16, C.byref(r))
    out = int(buf.value.decode(), 16)
    for z in (r, b, e, m):
        g.__gmpz_clear(C.byref(z))
    return out


def nlimbs(n: int) -> int:
    """kite_limbs(ctx) for exponent n: ceil((n + 64) / 64) words (reference src/ctx.c:241)."""
    return (n + 64 + 63) // 64


def limbs_digest(v: int, n: int) -> tuple[str, str]:
    b = v.to_bytes(8 * nlimbs(n), "little")
    return hashlib.sha256(b).hexdigest(), format(v & (2**64 - 1), "016X")


def seeded_k(seed: int, lo: int = 3, hi: int = 9999) -> int:
    rng = np.random.Generator(np.random.PCG64(seed))
    return int(rng.integers(lo // 2, hi // 2 + 1)) * 2 + 1


def seeded_residue(seed: int, k: int, n: int) -> int:
    """x0 uniform in [0, N): seeded 64-bit limbs reduced mod N."""
    N = k * (1 << n) - 1
    rng = np.random.Generator(np.random.PCG64(seed))
    words = rng.integers(0, 2**64, size=nlimbs(n), dtype=np.uint64)
    return int.from_bytes(words.astype("<u8").tobytes(), "little") % N


CHAINS = [
    # name, seed, k (None: seeded odd in [3, 9999]), n, squarings
    ("cpu_small", 101, 9357, 20000, 2000),
    ("cpu_mid", 102, None, 60000, 10000),
    ("single_28672", 1, None, 369717, 10000),
    ("single_49152", 2, None, 662695, 2000),
    ("mersenne_44497", 103, 1, 44497, 5000),
]

# the large single-test regime: k seeded odd in [3, 255], n seeded in [2e7, 2.5e7]
LARGE_CHAINS = [
    # name, seed, squarings
    ("large_a", 4, 100),
    ("large_b", 5, 100),
]

FERMAT = [
    # name, seed, n
    ("config1_full", 1, 369717),
    ("config2_full", 2, 662695),
]


def _chain(item):
    name, seed, k, n, count = item
    if k is None:
        k = seeded_k(seed)
    N = k * (1 << n) - 1
    x0 = seeded_residue(seed + 1000, k, n)
    v = gmp_powm(x0, 1 << count, N)
    sha, low = limbs_digest(v, n)
    return {"name": name, "seed": seed, "k": k, "n": n, "squarings": count,
            "x0_seed": seed + 1000, "sha256_limbs": sha, "low64": low}


def seeded_large(seed: int):
    rng = np.random.Generator(np.random.PCG64(seed))
    k = int(rng.integers(1, 128)) * 2 + 1          # odd in [3, 255]
    n = int(rng.integers(20_000_000, 25_000_001))
    return k, n


def _large_chain(item):
    name, seed, count = item
    k, n = seeded_large(seed)
    N = k * (1 << n) - 1
    x0 = seeded_residue(seed + 1000, k, n)
    v = gmp_powm(x0, 1 << count, N)
    sha, low = limbs_digest(v, n)
    return {"name": name, "seed": seed, "k": k, "n": n, "squarings": count,
            "x0_seed": seed + 1000, "sha256_limbs": sha, "low64": low}


def _fermat(item):
    name, seed, n = item
    k = seeded_k(seed)
    N = k * (1 << n) - 1
    r = gmp_powm(3, N - 1, N)
    return {"name": name, "seed": seed, "k": k, "n": n, "base": 3,
            "res64": format(r & (2**64 - 1), "016X"), "is_prp": r == 1}


def main(what: str) -> None:
    with ProcessPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        if what in ("chains", "all"):
            out = list(ex.map(_chain, CHAINS))
            with open(os.path.join(HERE, "chains.json"), "w") as f:
                json.dump(out, f, indent=1)
            print("chains.json written")
        if what in ("large", "all"):
            out = list(ex.map(_large_chain, LARGE_CHAINS))
            with open(os.path.join(HERE, "chains_large.json"), "w") as f:
                json.dump(out, f, indent=1)
            print("chains_large.json written")
        if what in ("fermat", "all"):
            out = list(ex.map(_fermat, FERMAT))
            with open(os.path.join(HERE, "fermat.json"), "w") as f:
                json.dump(out, f, indent=1)
            print("fermat.json written")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "all")
