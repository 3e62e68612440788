"""Many tests on the exact integer-NTT engine at once (include/kite_ntt.h, kn_group_*).

  python -m ahnum_gb300.ntt_group [--tests 256] [--squarings 64] [--reps 3] [--seed 3]

squares every test's number of the batched workload (k odd in [3, 10^4], n in [300000, 700000],
seeded PCG64, the benchmark's tests) `squarings` times per timed call and prints the GPU time per
squaring step of all tests (CUDA events on the group's stream) as one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import statistics

from . import native


class NttGroup:
    """A kn_group with one engine and one number per test, each number starting at 3."""

    def __init__(self, tests, device: int = 0, start: int = 3):
        self.lib = native.load()
        self.h = self.lib.kn_group_new(device)
        if not self.h:
            raise RuntimeError("kn_group_new failed")
        self.engines, self.nums = [], []
        try:
            for k, n in tests:
                e = self.lib.kn_engine_new(k, n, device)
                if not e:
                    raise RuntimeError(f"kn_engine_new({k}, {n}) failed")
                self.engines.append(e)
                x = self.lib.kn_num_alloc(e)
                if not x:
                    raise RuntimeError("kn_num_alloc failed")
                self.nums.append(x)
                limbs = (C.c_uint64 * self.lib.kn_limbs(e))()
                limbs[0] = start
                if self.lib.kn_set_limbs(e, x, limbs) != 0 or self.lib.kn_group_add(self.h, e, x) < 0:
                    raise RuntimeError("adding a test to the group failed")
        except Exception:
            self.close()
            raise

    def transform_lengths(self) -> dict:
        out = {}
        for e in self.engines:
            L = self.lib.kn_transform_len(e)
            out[L] = out.get(L, 0) + 1
        return dict(sorted(out.items()))

    def square(self, count: int) -> float:
        """Square every member `count` times; returns the GPU milliseconds of the call."""
        ms = C.c_float(0)
        if self.lib.kn_group_square(self.h, count, C.byref(ms)) != 0:
            raise RuntimeError(f"kn_group_square failed ({self.lib.kn_group_error(self.h)})")
        return ms.value

    def close(self):
        if self.h:
            self.lib.kn_group_free(self.h)
            self.h = None
        for e, x in zip(self.engines, self.nums):
            self.lib.kn_num_free(e, x)
        for e in self.engines:
            self.lib.kn_engine_free(e)
        self.engines, self.nums = [], []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def time_steps(tests, squarings: int = 64, reps: int = 3, device: int = 0):
    """(median seconds per squaring step of all tests, transform lengths)"""
    with NttGroup(tests, device) as g:
        g.square(16)  # graph capture, clocks
        times = [g.square(squarings) * 1e-3 / squarings for _ in range(reps)]
        return statistics.median(times), g.transform_lengths()


def main():
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ap = argparse.ArgumentParser()
    ap.add_argument("--tests", type=int, default=256)
    ap.add_argument("--squarings", type=int, default=64)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--seed", type=int, default=bench.SEED)
    args = ap.parse_args()
    tests = bench.workload(seed=args.seed, count=args.tests)
    t, lengths = time_steps(tests, args.squarings, args.reps)
    print(json.dumps({"tests": len(tests), "ms_per_squaring_step": t * 1e3,
                      "us_per_test_squaring": t * 1e6 / len(tests),
                      "transform_lengths": {str(k): v for k, v in lengths.items()}}))


if __name__ == "__main__":
    main()
