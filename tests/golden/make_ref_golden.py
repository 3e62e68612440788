"""Generates tests/golden/ref_backend.json from the reference's own `ref` backend.

The reference's portable backends are built from its sources by `make -C oracle ref
REF=<checkout>` (outputs in oracle/_ref/, git-ignored).  This script loads
oracle/_ref/libkiteref.so, runs the reference's public API on seeded inputs and records:

  squarings   for each (k, n, L): x0 uniform in [0, N) from random.Random(n), squared `count`
              times by kite_square_n on KITE_BACKEND_REF; the SHA-256 of the result's
              little-endian kite_limbs words, its low word, and kite_max_roundoff;
  lengths     kite_fft_len of a context made with fft_len 0 (the reference's length choice)
              for seeded (k, n) across the single-test, batched and served ranges.

The fixture lets the CPU suite and the GPU tests compare against the reference itself where the
reference checkout is absent.

Usage:  KITE_REFERENCE_SRC=<checkout> python tests/golden/make_ref_golden.py   (~1 min)
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

SQUARINGS = [
    # (k, n, L or 0 for the reference's choice, count)
    (9357, 20000, 0, 100),
    (1, 9941, 0, 100),
    (4095, 30000, 1920, 100),
    (3, 100000, 0, 100),
    (9357, 369717, 28672, 100),
    (9001, 662695, 49152, 40),
    (8243, 872226, 0, 20),
]


class _Opts(C.Structure):
    _fields_ = [("backend", C.c_int), ("fft_len", C.c_uint32), ("threads", C.c_uint32),
                ("plan_order", C.c_uint32)]


def _lib():
    from oracle import oracle
    if not os.path.exists(oracle.REF_LIB):
        oracle.build(ref=True)
    lib = C.CDLL(oracle.REF_LIB)
    vp = C.c_void_p
    lib.kite_ctx_new.restype = vp
    lib.kite_ctx_new.argtypes = [C.c_uint64, C.c_uint64, C.c_int32, vp]
    lib.kite_ctx_free.argtypes = [vp]
    lib.kite_num_new.restype = vp
    lib.kite_num_new.argtypes = [vp]
    lib.kite_num_free.argtypes = [vp, vp]
    lib.kite_set_limbs.argtypes = [vp, vp, C.POINTER(C.c_uint64)]
    lib.kite_get_limbs.argtypes = [vp, vp, C.POINTER(C.c_uint64)]
    lib.kite_square_n.argtypes = [vp, vp, C.c_uint64]
    lib.kite_limbs.restype = C.c_size_t
    lib.kite_limbs.argtypes = [vp]
    lib.kite_fft_len.restype = C.c_uint32
    lib.kite_fft_len.argtypes = [vp]
    lib.kite_max_roundoff.restype = C.c_double
    lib.kite_max_roundoff.argtypes = [vp]
    lib.kite_reset_roundoff.argtypes = [vp]
    return lib


def squarings(lib):
    out = []
    for k, n, L, count in SQUARINGS:
        o = _Opts(1, L, 0, 0)  # KITE_BACKEND_REF
        ctx = lib.kite_ctx_new(k, n, -1, C.byref(o))
        assert ctx, (k, n, L)
        try:
            Lr = lib.kite_fft_len(ctx)
            nl = lib.kite_limbs(ctx)
            N = k * (1 << n) - 1
            a = random.Random(n).randrange(N)
            x = lib.kite_num_new(ctx)
            arr = (C.c_uint64 * nl)(*[(a >> (64 * i)) & (2**64 - 1) for i in range(nl)])
            lib.kite_set_limbs(ctx, x, arr)
            lib.kite_reset_roundoff(ctx)
            lib.kite_square_n(ctx, x, count)
            res = (C.c_uint64 * nl)()
            lib.kite_get_limbs(ctx, x, res)
            err = lib.kite_max_roundoff(ctx)
            lib.kite_num_free(ctx, x)
        finally:
            lib.kite_ctx_free(ctx)
        v = sum(int(res[i]) << (64 * i) for i in range(nl))
        assert v == pow(a, 1 << count, N)
        out.append({"k": k, "n": n, "L": Lr, "count": count, "seed": n, "nlimbs": nl,
                    "sha256_limbs": hashlib.sha256(bytes(res)).hexdigest(), "low": f"{res[0]:016X}",
                    "maxerr": err})
        print(f"{k}*2^{n}-1 L={Lr}: {count} squarings, maxerr {err:.6f}", flush=True)
    return out


def lengths(lib):
    rng = random.Random(20251204)
    cases = []
    for lo, hi, klo, khi, cnt in [(300000, 700000, 3, 9999, 24), (100000, 4000000, 3, 9999, 16),
                                  (20000000, 25000000, 3, 255, 6), (2000, 90000, 1, 2**20, 12)]:
        for _ in range(cnt):
            k = rng.randrange(klo, khi + 1) | 1
            n = rng.randrange(lo, hi + 1)
            cases.append((k, n))
    out = []
    for k, n in cases:
        o = _Opts(1, 0, 0, 0)
        ctx = lib.kite_ctx_new(k, n, -1, C.byref(o))
        out.append({"k": k, "n": n, "L": lib.kite_fft_len(ctx) if ctx else 0})
        if ctx:
            lib.kite_ctx_free(ctx)
    return out


def main():
    lib = _lib()
    data = {"source": "reference kite, KITE_BACKEND_REF, built by `make -C oracle ref`",
            "squarings": squarings(lib), "lengths": lengths(lib)}
    with open(os.path.join(HERE, "ref_backend.json"), "w") as f:
        json.dump(data, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
