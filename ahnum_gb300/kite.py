"""Python mirror of the kite C API over libkite_gb300.so.

Same operations and argument meanings as the reference's include/kite.h (kite_ctx_new,
kite_num_new, kite_set_limbs/get_limbs, kite_square[_n], kite_mul, kite_mul_small, kite_add/sub,
kite_max_roundoff, kite_res64, kite_prp, kite_llr), with Python integers for values.  Every call
goes to the CUDA library; a missing library or GPU raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import native

CUDA = native.KITE_BACKEND_CUDA
CUDA_NTT = native.KITE_BACKEND_CUDA_NTT


def _limbs_from_int(v: int, nl: int):
    arr = (C.c_uint64 * nl)()
    b = v.to_bytes(8 * nl, "little")
    C.memmove(arr, b, 8 * nl)
    return arr


def _int_from_limbs(arr, nl: int) -> int:
    return int.from_bytes(C.string_at(arr, 8 * nl), "little")


class KiteError(RuntimeError):
    pass


class Num:
    """A number modulo N held on the GPU (kite_num)."""

    def __init__(self, ctx: "Ctx"):
        self.ctx = ctx
        self.h = ctx.lib.kite_num_new(ctx.h)
        if not self.h:
            raise KiteError("kite_num_new failed")

    def free(self):
        if self.h:
            self.ctx.lib.kite_num_free(self.ctx.h, self.h)
            self.h = None


class Ctx:
    """Context for N = k*2^n - 1 (kite_ctx) on the CUDA backend."""

    def __init__(self, k: int, n: int, fft_len: int = 0, backend: int = CUDA):
        self.lib = native.load()
        o = native.KiteOpts(backend, fft_len, 0, 0)
        self.h = self.lib.kite_ctx_new(k, n, -1, C.byref(o))
        if not self.h:
            raise KiteError(f"kite_ctx_new({k}, {n}, fft_len={fft_len}) failed")
        self.k, self.n = k, n
        self.N = k * (1 << n) - 1
        self.L = self.lib.kite_fft_len(self.h)
        self.nlimbs = self.lib.kite_limbs(self.h)
        self._nums = []

    def close(self):
        for x in self._nums:
            x.free()
        self._nums = []
        if self.h:
            self.lib.kite_ctx_free(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def num(self, value: int | None = None) -> Num:
        x = Num(self)
        self._nums.append(x)
        if value is not None:
            self.set(x, value)
        return x

    def set(self, x: Num, value: int):
        self.lib.kite_set_limbs(self.h, x.h, _limbs_from_int(value % self.N, self.nlimbs))

    def get(self, x: Num) -> int:
        arr = (C.c_uint64 * self.nlimbs)()
        self.lib.kite_get_limbs(self.h, x.h, arr)
        self.check()
        return _int_from_limbs(arr, self.nlimbs)

    def res64(self, x: Num) -> int:
        r = self.lib.kite_res64(self.h, x.h)
        self.check()
        return r

    def square(self, x: Num, count: int = 1):
        self.lib.kite_square_n(self.h, x.h, count)

    def mul(self, x: Num, y: Num):
        self.lib.kite_mul(self.h, x.h, y.h)

    def mul_small(self, x: Num, m: int):
        self.lib.kite_mul_small(self.h, x.h, m)

    def add(self, x: Num, y: Num):
        self.lib.kite_add(self.h, x.h, y.h)

    def sub(self, x: Num, y: Num):
        self.lib.kite_sub(self.h, x.h, y.h)

    def copy(self, dst: Num, src: Num):
        self.lib.kite_copy(self.h, dst.h, src.h)

    def maxerr(self) -> float:
        return self.lib.kite_max_roundoff(self.h)

    def reset_maxerr(self):
        self.lib.kite_reset_roundoff(self.h)

    def error(self) -> int:
        return self.lib.kite_ctx_error(self.h)

    def sync(self) -> int:
        return self.lib.kite_ctx_sync(self.h)

    def check(self):
        e = self.error()
        if e:
            raise KiteError(f"CUDA error {e} on context {self.k}*2^{self.n}-1")

    def corrupt(self, x: Num):
        self.lib.kite_debug_corrupt(self.h, x.h)


@dataclass
class PrpResult:
    rc: int
    res64: int
    is_prp: bool
    fft_len: int
    maxerr: float
    gerbicz_errors: int
    roundoff_retries: int
    resumed: bool
    resumed_at: int
    seconds: float


def prp(k: int, n: int, base: int = 3, fft_len: int = 0, gerbicz_block: int = 0,
        gerbicz_blocks: int = 0, inject_fault_at: int = 0, checkpoint: str | None = None,
        checkpoint_unverified: str | None = None, checkpoint_secs: float = 0.0,
        unverified_secs: float = 0.0, max_roundoff: float = 0.0, backend: int = CUDA) -> PrpResult:
    """kite_prp on a CUDA backend (the FP64 engine, or CUDA_NTT)."""
    lib = native.load()
    o = native.KitePrpOpts()
    o.fft = native.KiteOpts(backend, fft_len, 0, 0)
    o.gerbicz_block = gerbicz_block
    o.gerbicz_blocks = gerbicz_blocks
    o.max_roundoff = max_roundoff
    o.inject_fault_at = inject_fault_at
    o.checkpoint = checkpoint.encode() if checkpoint else None
    o.checkpoint_unverified = checkpoint_unverified.encode() if checkpoint_unverified else None
    o.checkpoint_secs = checkpoint_secs
    o.unverified_secs = unverified_secs
    r = native.KitePrpResult()
    rc = lib.kite_prp(k, n, base, C.byref(o), C.byref(r))
    return PrpResult(rc, r.res64, bool(r.is_prp), r.fft_len, r.maxerr, r.gerbicz_errors,
                     r.roundoff_retries, bool(r.resumed), r.resumed_at, r.seconds)


@dataclass
class LlrResult:
    rc: int
    is_prime: bool
    factor: int
    res64: int
    P: int
    fft_len: int
    maxerr: float
    roundoff_retries: int
    confirm_runs: int
    seconds: float


def llr(k: int, n: int, fft_len: int = 0, inject_fault_at: int = 0, inject_fault_runs: int = 0,
        inject_roundoff_at: int = 0, inject_roundoff_ladder: int = 0,
        checkpoint: str | None = None, backend: int = CUDA) -> LlrResult:
    """kite_llr on a CUDA backend (the FP64 engine, or CUDA_NTT)."""
    lib = native.load()
    o = native.KiteLlrOpts()
    o.fft = native.KiteOpts(backend, fft_len, 0, 0)
    o.inject_fault_at = inject_fault_at
    o.inject_fault_runs = inject_fault_runs
    o.inject_roundoff_at = inject_roundoff_at
    o.inject_roundoff_ladder = inject_roundoff_ladder
    o.checkpoint = checkpoint.encode() if checkpoint else None
    r = native.KiteLlrResult()
    rc = lib.kite_llr(k, n, C.byref(o), C.byref(r))
    return LlrResult(rc, bool(r.is_prime), r.factor, r.res64, r.P, r.fft_len, r.maxerr,
                     r.roundoff_retries, r.confirm_runs, r.seconds)


class Batch:
    """Many independent tests on one GPU (kc_batch_*): admit, step, collect."""

    def __init__(self, gerbicz_block: int = 1000, gerbicz_blocks: int = 0, mem_budget: int = 0,
                 device: int = -1):
        self.lib = native.load()
        self.h = self.lib.kc_batch_new(device, gerbicz_block, gerbicz_blocks, mem_budget)
        if not self.h:
            raise KiteError("kc_batch_new failed")
        self.gpu_ms = 0.0

    def close(self):
        if self.h:
            self.lib.kc_batch_free(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add_fermat(self, k: int, n: int, base: int = 3, fft_len: int = 0) -> int:
        return self.lib.kc_batch_add_fermat(self.h, k, n, base, fft_len)

    def add_llr(self, k: int, n: int, fft_len: int = 0) -> int:
        return self.lib.kc_batch_add_llr(self.h, k, n, fft_len)

    def step(self, blocks: int = 1) -> int:
        ms = C.c_double()
        r = self.lib.kc_batch_step(self.h, blocks, C.byref(ms))
        if r < 0:
            why = self.lib.kc_batch_error_string(self.h) or b""
            raise KiteError(f"kc_batch_step failed: {r} ({why.decode()})")
        self.gpu_ms += ms.value
        return r

    def result(self, slot: int):
        """(state, result): state 0 running, 1 done, 2 failed."""
        r = native.KcTestResult()
        st = self.lib.kc_batch_result(self.h, slot, C.byref(r))
        return st, r

    def release(self, slot: int):
        self.lib.kc_batch_release(self.h, slot)

    def active(self) -> int:
        return self.lib.kc_batch_active(self.h)

    def run(self, max_blocks: int = 1 << 30) -> None:
        blocks = 0
        while self.active() and blocks < max_blocks:
            self.step(1)
            blocks += 1
