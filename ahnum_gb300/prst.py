"""PRST-compatible Fermat proofs on the GB300 engine: the three proof operations of the
reference's `kite-prst` (tools/kite_prst.c:320-428, 511-555) as library calls.

  save(k, n, a, count, workdir)   Fermat test of k*2^n-1 to base a with count+1 proof points
                                  written as prst_<fp>.proof.<i>, then the products
                                  prst_<fp>.prod.<j>; returns the test result and the raw
                                  certificate RES64.
  build(k, n, a, count, workdir)  the certificate prst_<fp>.cert and its RES64.
  verify(k, n, path)              the certificate RES64 and M from squaring the certificate.

Every file matches the reference's byte for byte (include/kite_proof.h).  The test and all
proof arithmetic run on the GPU through libkite_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import native
from .kite import KiteError


@dataclass
class SaveResult:
    res64: int
    is_prp: bool
    fft_len: int
    maxerr: float
    raw_cert_res64: int
    prefix: str


def _lib():
    return native.load()


def prefix_for(k: int, n: int) -> str:
    return f"prst_{_lib().pp_fingerprint(k, n)}"


def points(n: int, count: int) -> list[int]:
    pos = (C.c_uint32 * (count + 1))()
    _lib().pp_points(n, count, pos)
    return list(pos)


def _ctx(k: int, n: int, fft_len: int = 0):
    lib = _lib()
    o = native.KiteOpts(native.KITE_BACKEND_CUDA, fft_len, 0, 0)
    ctx = lib.kite_ctx_new(k, n, -1, C.byref(o))
    if not ctx:
        raise KiteError(f"kite_ctx_new({k}, {n}) failed")
    return ctx


def save(k: int, n: int, a: int, count: int, workdir: str, keep: bool = False, fft_len: int = 0,
         gerbicz_block: int = 0) -> SaveResult:
    """The test with proof points, then the products (kite-prst -proof save COUNT [keep])."""
    if count < 2 or count & (count - 1):
        raise ValueError("proof count is not a power of 2")
    lib = _lib()
    prefix = os.path.join(workdir, prefix_for(k, n))
    fpP = lib.pp_proof_fingerprint(k, n, a)
    pos = (C.c_uint32 * (count + 1))()
    lib.pp_points(n, count, pos)
    failures = []

    def on_point(arg, index, it, limbs):
        # the full-length value trimmed to PRST's giant form
        nl = lib.kite_limbs(ctx)
        words = np.ctypeslib.as_array(limbs, shape=(nl,)).astype("<u8").view("<u4").copy()
        top = len(words)
        while top and words[top - 1] == 0:
            top -= 1
        g = native.PpGiant(words.ctypes.data_as(native.u32p), top)
        path = f"{prefix}.proof.{index}".encode()
        rc = lib.pp_write(path, native.PP_TYPE_VALUE, fpP, it, C.byref(g), 1)
        if rc:
            failures.append(path)
        return rc

    ctx = _ctx(k, n, fft_len)
    try:
        cb = native.POINT_FN(on_point)
        o = native.KitePrpOpts()
        o.fft = native.KiteOpts(native.KITE_BACKEND_CUDA, fft_len, 0, 0)
        o.gerbicz_block = gerbicz_block
        o.points = pos
        o.npoints = count + 1
        o.on_point = cb
        r = native.KitePrpResult()
        rc = lib.kite_prp(k, n, a, C.byref(o), C.byref(r))
        if rc or failures:
            raise KiteError(f"kite_prp with proof points failed ({rc}, {failures})")
        raw = C.c_uint64(0)
        rc = lib.pp_save_products(ctx, k, n, a, count, prefix.encode(), int(keep), None, C.byref(raw))
        if rc:
            raise KiteError(f"pp_save_products failed ({rc})")
        return SaveResult(r.res64, bool(r.is_prp), r.fft_len, r.maxerr, raw.value, prefix)
    finally:
        lib.kite_ctx_free(ctx)


def save_products(k: int, n: int, a: int, count: int, workdir: str, keep: bool = False,
                  abort: C.c_int | None = None) -> int:
    """Only the products, from points already on disk; returns the raw certificate RES64."""
    lib = _lib()
    prefix = os.path.join(workdir, prefix_for(k, n))
    ctx = _ctx(k, n)
    try:
        raw = C.c_uint64(0)
        rc = lib.pp_save_products(ctx, k, n, a, count, prefix.encode(), int(keep),
                                  C.byref(abort) if abort is not None else None, C.byref(raw))
        if rc:
            raise KiteError(f"pp_save_products failed ({rc})")
        return raw.value
    finally:
        lib.kite_ctx_free(ctx)


def build(k: int, n: int, a: int, count: int, workdir: str, keep: bool = False) -> int:
    """The certificate (kite-prst -proof build COUNT [keep]); returns its RES64."""
    lib = _lib()
    prefix = os.path.join(workdir, prefix_for(k, n))
    ctx = _ctx(k, n)
    try:
        res = C.c_uint64(0)
        rc = lib.pp_build_cert(ctx, k, n, a, count, prefix.encode(), int(keep), C.byref(res))
        if rc:
            raise KiteError(f"pp_build_cert failed ({rc})")
        return res.value
    finally:
        lib.kite_ctx_free(ctx)


def verify(k: int, n: int, path: str) -> tuple[int, int]:
    """(certificate RES64, M) of a certificate file (kite-prst -proof cert FILE)."""
    lib = _lib()
    ctx = _ctx(k, n)
    try:
        res, M = C.c_uint64(0), C.c_uint32(0)
        rc = lib.pp_verify_cert(ctx, k, n, path.encode(), C.byref(res), C.byref(M))
        if rc:
            raise KiteError(f"pp_verify_cert failed ({rc})")
        return res.value, M.value
    finally:
        lib.kite_ctx_free(ctx)
