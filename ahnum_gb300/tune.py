"""Per-length autotuner and round-off report (the GPU counterparts of the reference's
`kite tune`, tools/kite.c:274-326, and tools/sweep_err.c).

  python -m ahnum_gb300.tune shapes LMIN LMAX [--lengths L ...] [--out FILE]
      For every usable FFT length in [LMIN, LMAX] (multiples of 64 whose only prime factors are
      2, 3, 5, 7), time each candidate four-step shape H = R*C on a batch of tests of that length
      (batched throughput: microseconds per squaring per test, CUDA events) and keep the fastest.
      Writes "L us R C" lines; load them with kc_tuning_load or $KITE_GB300_TUNING.  The times
      also steer the length choice among safe lengths within 30 %, as the reference's tuning file
      does.

  python -m ahnum_gb300.tune roundoff L1 L2 ... [--k K] [--squarings S]
      For each length, the largest round-off over S squarings of a seeded residue at the largest
      n the reference's length model assigns to it for multiplier K (and at +0.25 and +0.5 bits
      per word beyond it), against the 0.4 limit the drivers enforce.
"""
from __future__ import annotations

import argparse
import ctypes as C
import math
import sys

from . import native
from .kite import Batch


def usable_lengths(lo: int, hi: int):
    out = []
    for L in range((lo + 63) // 64 * 64, hi + 1, 64):
        x = L
        for p in (2, 3, 5, 7):
            while x % p == 0:
                x //= p
        if x == 1:
            out.append(L)
    return out


def safe_bpw(L: int, k: int) -> float:
    """The reference's fitted model (src/ctx.c:26-33)."""
    return 21.44 - 0.305 * (math.log2(L) - 12) - 0.5 * math.log2(k) - 0.2


def time_shape(lib, L: int, R: int, slots: int, squarings: int) -> float:
    """Microseconds per squaring per test of a batch of `slots` tests at length L, shape R."""
    if lib.kc_set_fft_shape(L, R) != 0:
        return math.inf
    with Batch(gerbicz_block=squarings, gerbicz_blocks=1 << 20) as b:
        n = 12 * L
        for i in range(slots):
            if b.add_fermat(2 * i + 1, n, 3, L) < 0:
                return math.inf
        b.step(1)                 # graph capture, warm-up
        b.gpu_ms = 0.0
        b.step(2)
        return b.gpu_ms * 1e3 / (2 * squarings * slots)


def tune_shapes(lengths, slots: int = 48, squarings: int = 64, out=None, log=sys.stderr):
    lib = native.load()
    results = []
    Rs = (C.c_uint32 * 32)()
    Cs = (C.c_uint32 * 32)()
    for L in lengths:
        cnt = lib.kc_fft_shape_candidates(L, Rs, Cs, 32)
        best = (math.inf, 0, 0)
        for i in range(cnt):
            us = time_shape(lib, L, Rs[i], slots, squarings)
            print(f"  L={L} R={Rs[i]} C={Cs[i]}: {us:.3f} us/sq", file=log, flush=True)
            best = min(best, (us, Rs[i], Cs[i]))
        if best[1]:
            lib.kc_set_fft_shape(L, best[1])
            lib.kc_set_fft_time(L, best[0])
            results.append((L, best[0], best[1], best[2]))
            line = f"{L} {best[0]:.4f} {best[1]} {best[2]}"
            print(line, flush=True)
            if out:
                out.write(line + "\n")
                out.flush()
    return results


def roundoff_report(lengths, k: int = 9999, squarings: int = 500, seed: int = 1):
    lib = native.load()
    rows = []
    for L in lengths:
        row = [L]
        for extra in (0.0, 0.25, 0.5):
            n = int(L * (safe_bpw(L, k) + extra))
            e = lib.kc_roundoff_probe(k, n, L, squarings, seed)
            row.append((n, e))
        rows.append(row)
    return rows


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("shapes")
    a.add_argument("lmin", type=int)
    a.add_argument("lmax", type=int)
    a.add_argument("--lengths", type=int, nargs="*", help="tune only these lengths in the range")
    a.add_argument("--out")
    a.add_argument("--slots", type=int, default=48)
    a.add_argument("--squarings", type=int, default=64)
    b = sub.add_parser("roundoff")
    b.add_argument("lengths", type=int, nargs="+")
    b.add_argument("--k", type=int, default=9999)
    b.add_argument("--squarings", type=int, default=500)
    args = ap.parse_args()
    if args.cmd == "shapes":
        out = open(args.out, "w") if args.out else None
        try:
            Ls = usable_lengths(args.lmin, args.lmax)
            if args.lengths:
                Ls = [L for L in Ls if L in set(args.lengths)]
            tune_shapes(Ls, args.slots, args.squarings, out)
        finally:
            if out:
                out.close()
    else:
        print("| L | n at model limit | maxerr | n at +0.25 bit | maxerr | n at +0.5 bit | maxerr |")
        print("|---|---|---|---|---|---|---|")
        for L, (n0, e0), (n1, e1), (n2, e2) in roundoff_report(args.lengths, args.k, args.squarings):
            print(f"| {L} | {n0} | {e0:.4f} | {n1} | {e1:.4f} | {n2} | {e2:.4f} |", flush=True)


if __name__ == "__main__":
    main()
