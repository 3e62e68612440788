"""Per-length autotuner and round-off report (the GPU counterparts of the reference's
`kite tune`, tools/kite.c:274-326, and tools/sweep_err.c).

  python -m ahnum_gb300.tune shapes LMIN LMAX [--lengths L ...] [--out FILE]
      For every usable FFT length in [LMIN, LMAX] (multiples of 64 whose only prime factors are
      2, 3, 5, 7), time each candidate four-step shape H = R*C on a batch of tests of that length
      (batched throughput: microseconds per squaring per test, CUDA events) and keep the fastest.
      Writes "L us R C" lines; load them with kc_tuning_load or $KITE_GB300_TUNING.  The times
      also steer the length choice among safe lengths within 30 %, as the reference's tuning file
      does.

  python -m ahnum_gb300.tune latency K:N [K:N ...] [--out FILE]
      For each number, at the length the reference's chooser gives it: time every usable
      four-step shape H = R*C with every column-group width G in {2, 4, 8} for one test run alone
      (kc_engine_new, squarings queued back to back, wall clock around them) and keep the
      fastest.  Writes "L us R C G" lines (kc_tuning_load reads them as latency shapes); the
      built-in model's own choice is timed first and kept unless a shape beats it.

  python -m ahnum_gb300.tune roundoff L1 L2 ... [--k K] [--squarings S]
      For each length, the largest round-off over S squarings of a seeded residue at the largest
      n the reference's length model assigns to it for multiplier K (and at +0.25 and +0.5 bits
      per word beyond it), against the 0.4 limit the drivers enforce.
"""
from __future__ import annotations

import argparse
import ctypes as C
import math
import os
import sys

from . import native
from .kite import Batch


HERE = os.path.dirname(os.path.abspath(__file__))
THROUGHPUT_FILE = os.path.join(HERE, "tuning_gb300.txt")
LATENCY_FILE = os.path.join(HERE, "tuning_gb300_latency.txt")


def load_gb300_tuning(lib) -> None:
    """Applies the shipped GB300 shapes: the batched four-step shapes (shapes only: the FFT
    lengths stay the ones the reference's length chooser picks without a times file) and the
    single-test latency shapes."""
    if os.path.exists(THROUGHPUT_FILE):
        with open(THROUGHPUT_FILE) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 4 and not line.startswith("#"):
                    lib.kc_set_fft_shape(int(parts[0]), int(parts[2]))
    if os.path.exists(LATENCY_FILE):
        with open(LATENCY_FILE) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 5 and not line.startswith("#"):
                    lib.kc_set_latency_shape(int(parts[0]), int(parts[2]), int(parts[4]))


def unload_gb300_tuning(lib) -> None:
    """Returns every length of the shipped files to the built-in shapes (engines made afterwards
    use them; plans already built keep theirs)."""
    for path, reset in ((THROUGHPUT_FILE, lambda L: lib.kc_set_fft_shape(L, 0)),
                        (LATENCY_FILE, lambda L: lib.kc_set_latency_shape(L, 0, 0))):
        if not os.path.exists(path):
            continue
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) in (4, 5) and not line.startswith("#"):
                    reset(int(parts[0]))


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


def latency_shapes(L: int):
    """Every usable (R, C) of H = L/2 for a test run alone: C a multiple of 8 in [16, 2048],
    R in [2, 1024], both with prime factors 2, 3, 5, 7 only."""
    H = L // 2
    out = []
    for c in range(16, 2049, 8):
        if H % c:
            continue
        r = H // c
        if 2 <= r <= 1024 and all(_smooth(v) for v in (r, c)):
            out.append((r, c))
    return out


def _smooth(v: int) -> bool:
    for p in (2, 3, 5, 7):
        while v % p == 0:
            v //= p
    return v == 1


def time_latency(lib, k: int, n: int, L: int, squarings: int, warmup: int = 20):
    """(microseconds per squaring, R, C, G) of one test alone with the shape the library picks
    now; None if the engine cannot be made."""
    import time
    e = lib.kc_engine_new(k, n, L, None, None, None, 0, 0, 0, 0, -1)
    if not e:
        return None
    try:
        R, Cc = C.c_uint32(), C.c_uint32()
        lib.kc_shape(e, C.byref(R), C.byref(Cc))
        G = lib.kc_group_width(e)
        x = lib.kc_num_alloc(e)
        digits = (C.c_int64 * L)()
        digits[0] = 3
        if not x or lib.kc_from_digits(e, x, digits) != 0:
            return None
        lib.kc_square(e, x, warmup)
        lib.kc_sync(e)
        t0 = time.perf_counter()
        lib.kc_square(e, x, squarings)
        rc = lib.kc_sync(e)
        dt = time.perf_counter() - t0
        lib.kc_num_free(e, x)
        if rc != 0:
            return None
        return dt / squarings * 1e6, R.value, Cc.value, G
    finally:
        lib.kc_engine_free(e)


def tune_latency(numbers, squarings: int = 200, out=None, log=sys.stderr):
    lib = native.load()
    results = []
    for k, n in numbers:
        L = lib.kc_choose_fft_len(k, n)
        lib.kc_set_latency_shape(L, 0, 0)
        model = time_latency(lib, k, n, L, squarings)
        if model is None:
            print(f"  {k}*2^{n}-1: no engine at L={L}", file=log, flush=True)
            continue
        print(f"  L={L} model R={model[1]} C={model[2]} G={model[3]}: {model[0]:.2f} us/sq",
              file=log, flush=True)
        best = model
        for R, Cc in latency_shapes(L):
            for G in (2, 4, 8):
                if Cc % G or lib.kc_set_latency_shape(L, R, G) != 0:
                    continue
                t = time_latency(lib, k, n, L, squarings)
                lib.kc_set_latency_shape(L, 0, 0)
                if t is None or (t[1], t[3]) != (R, G):
                    continue  # this number's digits do not allow groups of G
                print(f"  L={L} R={R} C={Cc} G={G}: {t[0]:.2f} us/sq", file=log, flush=True)
                best = min(best, t)
        lib.kc_set_latency_shape(L, best[1], best[3])
        results.append((L,) + best)
        line = f"{L} {best[0]:.3f} {best[1]} {best[2]} {best[3]}"
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


def bpw_limit(lib, L: int, k: int, threshold: float, squarings: int, seed: int = 1, step: float = 0.05) -> float:
    """The largest bits per word (to `step`) at which the round-off of `squarings` squarings of a
    seeded residue at length L stays at or below `threshold`: the reference's fitting method
    (tools/fit_bpw.py, bisection from its model's guess), run on these kernels."""
    guess = (53 - 6 - 0.5 * math.log2(L) - math.log2(k)) / 2
    lo, hi = guess - 3, guess + 4
    while hi - lo > step:
        mid = (lo + hi) / 2
        e = lib.kc_roundoff_probe(k, int(mid * L), L, squarings, seed)
        if 0 <= e <= threshold:
            lo = mid
        else:
            hi = mid
    return lo


def fit_bpw(lengths, ks, threshold: float = 0.25, squarings: int = 300):
    """bpw_limit over a grid of lengths and multipliers, and the least-squares fit of the
    reference's model form bpw = a - b (log2 L - 12) - c log2 k.  Returns (rows, (a, b, c))."""
    import numpy as np
    lib = native.load()
    rows = []
    for L in lengths:
        for k in ks:
            rows.append((L, k, bpw_limit(lib, L, k, threshold, squarings)))
    A = np.array([[1.0, -(math.log2(L) - 12), -math.log2(k)] for L, k, _ in rows])
    y = np.array([b for _, _, b in rows])
    coef = np.linalg.lstsq(A, y, rcond=None)[0]
    return rows, tuple(float(v) for v in coef)


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
    c = sub.add_parser("latency")
    c.add_argument("numbers", nargs="+", help="K:N pairs")
    c.add_argument("--squarings", type=int, default=200)
    c.add_argument("--out")
    f = sub.add_parser("fp64", help="the FP64 probe in several shapes and opcodes (lane ops per second)")
    f.add_argument("--device", type=int, default=0)
    g = sub.add_parser("fitbpw", help="fit the safe bits-per-word model to these kernels")
    g.add_argument("--lengths", type=int, nargs="+",
                   default=[4096, 16384, 20480, 24576, 28672, 32768, 36864, 40960, 49152, 65536, 262144, 1048576])
    g.add_argument("--ks", type=int, nargs="+", default=[1, 3, 31, 255, 2047, 9999])
    g.add_argument("--threshold", type=float, default=0.25)
    g.add_argument("--squarings", type=int, default=300)
    b = sub.add_parser("roundoff")
    b.add_argument("lengths", type=int, nargs="+")
    b.add_argument("--k", type=int, default=9999)
    b.add_argument("--squarings", type=int, default=500)
    args = ap.parse_args()
    if args.cmd == "fp64":
        lib = native.load()
        print("| opcode | chains per thread | blocks per SM x threads | G lane ops/s | TFLOP/s (FMA = 2) |")
        print("|---|---|---|---|---|")
        for op, chains, bps, thr in ((0, 8, 4, 256), (0, 8, 8, 256), (0, 16, 4, 256), (0, 16, 8, 256),
                                     (0, 4, 8, 256), (0, 8, 2, 256), (0, 8, 16, 128), (1, 8, 8, 256),
                                     (2, 8, 8, 256)):
            r = lib.kc_fp64_probe_rate(args.device, bps, thr, chains, op)
            name = ("DFMA", "DMUL", "DADD")[op]
            tf = f"{2 * r / 1e12:.4f}" if op == 0 else "-"
            print(f"| {name} | {chains} | {bps} x {thr} | {r / 1e9:.1f} | {tf} |", flush=True)
        return
    if args.cmd == "fitbpw":
        rows, (a, b_, c) = fit_bpw(args.lengths, args.ks, args.threshold, args.squarings)
        print(f"| L | k | largest bpw with maxerr <= {args.threshold} over {args.squarings} squarings | "
              "reference model without its 0.2 margin |")
        print("|---|---|---|---|")
        for L, k, bpw in rows:
            ref = safe_bpw(L, k) + 0.2
            print(f"| {L} | {k} | {bpw:.2f} | {ref:.2f} |", flush=True)
        print(f"\nfit: bpw = {a:.3f} - {b_:.4f} (log2 L - 12) - {c:.4f} log2 k   "
              f"(reference: 21.44 - 0.305 (log2 L - 12) - 0.5 log2 k, then 0.2 below)")
        return
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
    elif args.cmd == "latency":
        out = open(args.out, "w") if args.out else None
        try:
            nums = [tuple(int(v) for v in a.split(":")) for a in args.numbers]
            tune_latency(nums, args.squarings, out)
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
