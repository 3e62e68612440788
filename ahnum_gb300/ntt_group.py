"""Many tests on the exact integer-NTT engine at once (include/kite_ntt.h, kn_group_*).

  python -m ahnum_gb300.ntt_group [--tests 256] [--squarings 64] [--reps 3] [--seed 3] [--streams 2]

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


def split_members(members, parts: int, size=lambda m: m):
    """`members` dealt into `parts` lists of about equal work, largest first."""
    order = sorted(members, key=size, reverse=True)
    out = [[] for _ in range(max(1, min(parts, len(order))))]
    load = [0] * len(out)
    for m in order:
        i = load.index(min(load))
        out[i].append(m)
        load[i] += size(m)
    return out


def square_groups(lib, groups, count: int) -> float:
    """kn_groups_square of several groups (one stream each); returns the GPU milliseconds."""
    arr = (C.c_void_p * len(groups))(*groups)
    ms = C.c_float(0)
    if lib.kn_groups_square(arr, len(groups), count, C.byref(ms)) != 0:
        raise RuntimeError("kn_groups_square failed")
    return ms.value


class NttGroup:
    """One engine and one number per test, each number starting at 3, in `streams` kn_groups of
    about equal work that square together, one CUDA stream each."""

    def __init__(self, tests, device: int = 0, start: int = 3, streams: int = 2):
        self.lib = native.load()
        self.engines, self.nums, self.groups = [], [], []
        try:
            parts = split_members(list(enumerate(tests)), streams, size=lambda m: m[1][1])
            member_group = {}
            for gi, part in enumerate(parts):
                g = self.lib.kn_group_new(device)
                if not g:
                    raise RuntimeError("kn_group_new failed")
                self.groups.append(g)
                for i, _ in part:
                    member_group[i] = g
            for i, (k, n) in enumerate(tests):
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
                if self.lib.kn_set_limbs(e, x, limbs) != 0 or self.lib.kn_group_add(member_group[i], e, x) < 0:
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
        return square_groups(self.lib, self.groups, count)

    def close(self):
        for g in self.groups:
            self.lib.kn_group_free(g)
        self.groups = []
        for e, x in zip(self.engines, self.nums):
            self.lib.kn_num_free(e, x)
        for e in self.engines:
            self.lib.kn_engine_free(e)
        self.engines, self.nums = [], []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def residue_nm1(y: int, N: int, base: int) -> int:
    """base^(N+1) mod N -> base^(N-1) mod N, also when base and N share a factor (the
    reference's kite_residue_nm1, src/prp.c:63-144): N = Q*M with Q made of the primes of base;
    the result is 0 mod Q and y / base^2 mod M, joined by the CRT."""
    q, b, m = 1, base, N
    p = 2
    while b > 1:
        if b % p == 0:
            while b % p == 0:
                b //= p
            while m % p == 0:
                if q > 1 << 40:
                    raise ValueError("the base-prime part of N does not fit a word")
                q *= p
                m //= p
        p += 1
    if q == 1:
        return y * pow(base * base, -1, N) % N
    t = y % m * pow(base * base, -1, m) % m
    u = -t * pow(m, -1, q) % q
    return t + m * u


class NttFermatBatch:
    """Fermat base-a PRP tests of many N = k*2^n-1 on the integer-NTT engine, in lockstep Gerbicz
    blocks: every block squares all tests' x B times (`streams` groups of about equal work, one
    CUDA stream each, one launch set per group per squaring) and
    multiplies d <- d*x (one group product); every M blocks, t = d before the block's product is
    checked as x0 * t^(2^B) == d, the reference's check (src/prp.c:407-567), and the verified
    (x, d) kept on the host; a failed check returns every test to its verified state.  A test
    whose remaining squarings fall below a block leaves the group and finishes alone with a
    doubled tail (the tail squared twice and compared), as kite_prp does."""

    def __init__(self, tests, base: int = 3, block: int = 1000, blocks_per_check: int = 250,
                 device: int = 0, streams: int = 2):
        self.lib = native.load()
        self.base, self.B, self.M, self.device = base, block, blocks_per_check, device
        self.streams = streams   # the block squarings run as this many groups, one stream each
        self.t = []
        for k, n in tests:
            e = self.lib.kn_engine_new(k, n, device)
            if not e:
                self.close()
                raise RuntimeError(f"kn_engine_new({k}, {n}) failed")
            N = k * (1 << n) - 1
            st = {"k": k, "n": n, "N": N, "e": e, "nl": self.lib.kn_limbs(e), "done": 0,
                  "res64": None, "is_prp": None, "gerbicz_errors": 0}
            for name in ("x", "d", "t", "x0"):
                st[name] = self.lib.kn_num_alloc(e)
            x0 = pow(base, k, N)
            for name in ("x", "d", "x0"):
                self._set(st, name, x0)
            st["vx"] = st["vd"] = x0
            self.t.append(st)
        self.gpu_ms = 0.0        # GPU time of every group operation
        self.block_ms = 0.0      # of the blocks alone (B squarings and the product), checks excluded
        self.blocks = 0
        self.fault = None        # (k, squarings done): corrupt that test's x once, for tests

    def _set(self, st, name, v):
        arr = (C.c_uint64 * st["nl"])()
        C.memmove(arr, v.to_bytes(8 * st["nl"], "little"), 8 * st["nl"])
        if self.lib.kn_set_limbs(st["e"], st[name], arr) != 0:
            raise RuntimeError("kn_set_limbs failed")

    def _get(self, st, name) -> int:
        arr = (C.c_uint64 * st["nl"])()
        if self.lib.kn_get_limbs(st["e"], st[name], arr) != 0:
            raise RuntimeError("kn_get_limbs failed")
        return int.from_bytes(C.string_at(arr, 8 * st["nl"]), "little")

    def _group(self, members, which):
        g = self.lib.kn_group_new(self.device)
        for st in members:
            if self.lib.kn_group_add(g, st["e"], st[which]) < 0:
                raise RuntimeError("kn_group_add failed")
        return g

    def _timed(self, rc, ms):
        if rc != 0:
            raise RuntimeError("kn_group operation failed")
        self.gpu_ms += ms.value

    def _square(self, g, count):
        ms = C.c_float(0)
        self._timed(self.lib.kn_group_square(g, count, C.byref(ms)), ms)

    def _square_groups(self, groups, count):
        self.gpu_ms += square_groups(self.lib, groups, count)

    def _mul(self, g, members, which):
        ys = (C.c_void_p * len(members))(*[st[which] for st in members])
        ms = C.c_float(0)
        self._timed(self.lib.kn_group_mul(g, ys, C.byref(ms)), ms)

    def _finish(self, st):
        """the last squarings (fewer than a block) twice, compared; then the residue"""
        rest = st["n"] - st["done"]
        e = st["e"]
        self.lib.kn_copy(e, st["t"], st["x"])
        self.lib.kn_square(e, st["x"], rest)
        self.lib.kn_square(e, st["t"], rest)
        a, b = self._get(st, "x"), self._get(st, "t")
        if a != b:
            raise RuntimeError("tail mismatch")
        N = st["N"]
        r = residue_nm1(a, N, self.base)
        st["res64"] = r & (2**64 - 1)
        st["is_prp"] = a == self.base * self.base
        st["done"] = st["n"]

    def run(self, max_blocks: int | None = None):
        """Runs the tests to their residues (or `max_blocks` blocks); returns the results."""
        blocks = 0
        while True:
            active = [st for st in self.t if st["res64"] is None and st["n"] - st["done"] >= self.B]
            for st in self.t:
                if st["res64"] is None and st not in active:
                    self._finish(st)
            if not active or (max_blocks is not None and blocks >= max_blocks):
                break
            gxs = [self._group(part, "x")
                   for part in split_members(active, self.streams, size=lambda st: st["n"])]
            gd, gt = (self._group(active, w) for w in ("d", "t"))
            try:
                # blocks until the next check, or until a test would leave the lockstep
                room = min((st["n"] - st["done"]) // self.B for st in active)
                span = min(self.M, room)
                if max_blocks is not None:
                    span = min(span, max_blocks - blocks)
                for j in range(span):
                    if j == span - 1:
                        for st in active:
                            self.lib.kn_copy(st["e"], st["t"], st["d"])
                    before = self.gpu_ms
                    self._square_groups(gxs, self.B)
                    for st in active:
                        st["done"] += self.B
                        if self.fault and self.fault[0] == st["k"] and st["done"] == self.fault[1]:
                            self._corrupt(st)
                            self.fault = None
                    self._mul(gd, active, "x")
                    self.block_ms += self.gpu_ms - before
                    self.blocks += 1
                blocks += span
                # check: x0 * t^(2^B) == d
                self._square(gt, self.B)
                self._mul(gt, active, "x0")
                for st in active:
                    if self._get(st, "t") == self._get(st, "d"):
                        st["vx"], st["vd"], st["vdone"] = self._get(st, "x"), self._get(st, "d"), st["done"]
                    else:
                        st["gerbicz_errors"] += 1
                        self._set(st, "x", st["vx"])
                        self._set(st, "d", st["vd"])
                        st["done"] = st.get("vdone", 0)
            finally:
                for g in gxs + [gd, gt]:
                    self.lib.kn_group_free(g)
        return [{"k": st["k"], "n": st["n"], "res64": st["res64"], "is_prp": st["is_prp"],
                 "gerbicz_errors": st["gerbicz_errors"]} for st in self.t]

    def _corrupt(self, st):
        v = self._get(st, "x")
        self._set(st, "x", (v + (1 << (st["n"] // 3))) % st["N"])

    def close(self):
        for st in self.t:
            for name in ("x", "d", "t", "x0"):
                if st.get(name):
                    self.lib.kn_num_free(st["e"], st[name])
            self.lib.kn_engine_free(st["e"])
        self.t = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def time_steps(tests, squarings: int = 64, reps: int = 3, device: int = 0, streams: int = 2):
    """(median seconds per squaring step of all tests, transform lengths)"""
    with NttGroup(tests, device, streams=streams) as g:
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
    ap.add_argument("--streams", type=int, default=2, help="groups squared together, one stream each")
    args = ap.parse_args()
    tests = bench.workload(seed=args.seed, count=args.tests)
    t, lengths = time_steps(tests, args.squarings, args.reps, streams=args.streams)
    print(json.dumps({"tests": len(tests), "streams": args.streams, "ms_per_squaring_step": t * 1e3,
                      "us_per_test_squaring": t * 1e6 / len(tests),
                      "transform_lengths": {str(k): v for k, v in lengths.items()}}))


if __name__ == "__main__":
    main()
