"""ctypes binding of the CPU oracle (kite_oracle.c) and, when built, the reference's own
portable backends (oracle/_ref/libkiteref.so).  TEST INFRASTRUCTURE ONLY: used by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libkite_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libkiteref.so")
REF_CLI = os.path.join(HERE, "_ref", "kite")
# The reference checkout, for building its portable backends (`make ref`): taken from the
# environment, as the checkout exists only where the fixtures are made, never on a GPU host.
REFERENCE_SRC = os.environ.get("KITE_REFERENCE_SRC", "")

u64p = C.POINTER(C.c_uint64)
dp = C.POINTER(C.c_double)
vp = C.c_void_p

_lock = threading.Lock()
_lib = None


def build(ref: bool | None = None) -> None:
    """make the oracle; also the reference backends when $KITE_REFERENCE_SRC names a checkout."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    have_src = bool(REFERENCE_SRC) and os.path.isdir(os.path.join(REFERENCE_SRC, "src"))
    if ref is None:
        ref = have_src
    if ref and have_src:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_SRC}"], check=True)


def load():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(ORACLE_LIB):
                build(ref=False)
            lib = C.CDLL(ORACLE_LIB)
            sig = {
                "ko_fft_len_ok": (C.c_int, [C.c_uint32]),
                "ko_safe_bpw": (C.c_double, [C.c_uint32, C.c_uint64]),
                "ko_choose_fft_len": (C.c_uint32, [C.c_uint64, C.c_uint64]),
                "ko_next_fft_len": (C.c_uint32, [C.c_uint32]),
                "ko_ctx_new": (vp, [C.c_uint64, C.c_uint64, C.c_uint32]),
                "ko_ctx_free": (None, [vp]),
                "ko_fft_len": (C.c_uint32, [vp]),
                "ko_limbs": (C.c_size_t, [vp]),
                "ko_layout": (None, [vp, C.POINTER(C.c_uint8), dp, dp, u64p]),
                "ko_set_limbs": (None, [vp, dp, u64p]),
                "ko_get_limbs": (None, [vp, dp, u64p]),
                "ko_res64": (C.c_uint64, [vp, dp]),
                "ko_digits_to_limbs": (None, [vp, C.POINTER(C.c_int64), u64p]),
                "ko_carry_digits": (None, [vp, C.POINTER(C.c_int64)]),
                "ko_square": (None, [vp, dp, C.c_uint64]),
                "ko_mul": (None, [vp, dp, dp]),
                "ko_mul_small": (None, [vp, dp, C.c_int64]),
                "ko_add": (None, [vp, dp, dp]),
                "ko_sub": (None, [vp, dp, dp]),
                "ko_maxerr": (C.c_double, [vp]),
                "ko_reset_maxerr": (None, [vp]),
                "ko_residue_nm1": (C.c_int, [u64p, u64p, C.c_size_t, C.c_uint64]),
                "ko_fermat": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, u64p,
                                        C.POINTER(C.c_int), dp]),
                "ko_llr_choose_P": (C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint32), u64p]),
                "ko_llr": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, C.POINTER(C.c_uint32),
                                     u64p, u64p, C.POINTER(C.c_int), dp]),
                "ko_time_squarings": (C.c_int, [u64p, u64p, C.POINTER(C.c_uint32), C.c_int, C.c_int,
                                                C.c_uint32, dp]),
            }
            for name, (res, args) in sig.items():
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            _lib = lib
        return _lib


def _limbs(v: int, nl: int):
    a = (C.c_uint64 * nl)()
    C.memmove(a, v.to_bytes(8 * nl, "little"), 8 * nl)
    return a


def _int(a, nl: int) -> int:
    return int.from_bytes(C.string_at(a, 8 * nl), "little")


class OracleCtx:
    """The oracle's context: numbers are Python-held arrays of L digit doubles."""

    def __init__(self, k: int, n: int, L: int = 0):
        self.lib = load()
        self.h = self.lib.ko_ctx_new(k, n, L)
        if not self.h:
            raise ValueError(f"oracle cannot lay out {k}*2^{n}-1 at L={L}")
        self.k, self.n = k, n
        self.N = k * (1 << n) - 1
        self.L = self.lib.ko_fft_len(self.h)
        self.nlimbs = self.lib.ko_limbs(self.h)

    def close(self):
        if self.h:
            self.lib.ko_ctx_free(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def num(self, value: int = 0):
        x = (C.c_double * self.L)()
        self.set(x, value)
        return x

    def set(self, x, value: int):
        self.lib.ko_set_limbs(self.h, x, _limbs(value % self.N, self.nlimbs))

    def get(self, x) -> int:
        a = (C.c_uint64 * self.nlimbs)()
        self.lib.ko_get_limbs(self.h, x, a)
        return _int(a, self.nlimbs)

    def square(self, x, count: int = 1):
        self.lib.ko_square(self.h, x, count)

    def mul(self, x, y):
        self.lib.ko_mul(self.h, x, y)

    def mul_small(self, x, m: int):
        self.lib.ko_mul_small(self.h, x, m)

    def add(self, x, y):
        self.lib.ko_add(self.h, x, y)

    def sub(self, x, y):
        self.lib.ko_sub(self.h, x, y)

    def maxerr(self) -> float:
        return self.lib.ko_maxerr(self.h)

    def reset_maxerr(self):
        self.lib.ko_reset_maxerr(self.h)

    def layout(self):
        L = self.L
        bits = (C.c_uint8 * L)()
        w = (C.c_double * L)()
        osc = (C.c_double * L)()
        meta = (C.c_uint64 * 5)()
        self.lib.ko_layout(self.h, bits, w, osc, meta)
        return bytes(bits), list(w), list(osc), list(meta)

    def digits_to_int(self, digits) -> int:
        d = (C.c_int64 * self.L)(*digits)
        a = (C.c_uint64 * self.nlimbs)()
        self.lib.ko_digits_to_limbs(self.h, d, a)
        return _int(a, self.nlimbs)


def fermat(k: int, n: int, base: int = 3, L: int = 0):
    lib = load()
    r = C.c_uint64()
    p = C.c_int()
    e = C.c_double()
    rc = lib.ko_fermat(k, n, base, L, C.byref(r), C.byref(p), C.byref(e))
    return rc, r.value, bool(p.value), e.value


def llr(k: int, n: int, L: int = 0):
    lib = load()
    P = C.c_uint32()
    f = C.c_uint64()
    r = C.c_uint64()
    pr = C.c_int()
    e = C.c_double()
    rc = lib.ko_llr(k, n, L, C.byref(P), C.byref(f), C.byref(r), C.byref(pr), C.byref(e))
    return rc, P.value, f.value, r.value, bool(pr.value), e.value


def choose_fft_len(k: int, n: int) -> int:
    return load().ko_choose_fft_len(k, n)


def time_squarings(tests, threads: int, squarings: int):
    """tests: list of (k, n, L); returns microseconds per squaring for each test."""
    lib = load()
    m = len(tests)
    ks = (C.c_uint64 * m)(*[t[0] for t in tests])
    ns = (C.c_uint64 * m)(*[t[1] for t in tests])
    Ls = (C.c_uint32 * m)(*[t[2] for t in tests])
    us = (C.c_double * m)()
    lib.ko_time_squarings(ks, ns, Ls, m, threads, squarings, us)
    return list(us)
