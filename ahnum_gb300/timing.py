"""Time one test's squarings on the GPU (the single-test path the reference's `kite time`
measures on the CPU, tools/kite.c).

  python -m ahnum_gb300.timing K N [--fft-len L] [--squarings S] [--warmup W] [--backend cuda|cuda-ntt]

squares 3 modulo N = K*2^N-1 W times, then S times, and prints the microseconds per squaring
(wall clock around kite_square_n, synchronised) with the transform length and round-off as one
JSON line.  The shipped GB300 shapes (ahnum_gb300/tuning_gb300*.txt) are applied first.
"""
from __future__ import annotations

import argparse
import json
import time

from . import native
from .kite import CUDA, CUDA_NTT, Ctx
from .tune import load_gb300_tuning


def time_single(k: int, n: int, fft_len: int = 0, squarings: int = 200, warmup: int = 20,
                backend: int = CUDA) -> dict:
    load_gb300_tuning(native.load())
    with Ctx(k, n, fft_len, backend=backend) as c:
        x = c.num(3)
        c.square(x, warmup)
        c.sync()
        t0 = time.perf_counter()
        c.square(x, squarings)
        c.sync()
        dt = time.perf_counter() - t0
        return {"k": k, "n": n, "fft_len": c.L, "squarings": squarings,
                "us_per_squaring": dt / squarings * 1e6, "maxerr": c.maxerr(),
                "backend": "cuda-ntt" if backend == CUDA_NTT else "cuda"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("k", type=int)
    ap.add_argument("n", type=int)
    ap.add_argument("--fft-len", type=int, default=0)
    ap.add_argument("--squarings", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--backend", choices=["cuda", "cuda-ntt"], default="cuda")
    a = ap.parse_args()
    print(json.dumps(time_single(a.k, a.n, a.fft_len, a.squarings, a.warmup,
                                 CUDA_NTT if a.backend == "cuda-ntt" else CUDA)))


if __name__ == "__main__":
    main()
