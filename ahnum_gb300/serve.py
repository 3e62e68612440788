"""Served request loop: Fermat and LLR tests admitted into one running GPU batch as they arrive.

Requests arrive over time (a seeded Poisson stream by default: 80 % Fermat base 3, 20 % LLR,
k uniform odd in [3, 10^4], n log-uniform in [10^5, 4*10^6]).  The loop admits every waiting
request the device-memory budget allows into the kc_batch (kc_batch_add_* refuses with -2 when
it is full), advances all admitted tests together one Gerbicz block at a time, releases each
slot as soon as its verdict is in, and admits the next requests into the freed memory while
the others keep running.  That is continuous batching, not a queue: work that arrives while
other tests are on the GPU overlaps with them on the device.

Per test: the Fermat verdict is the batch's Gerbicz-checked result (the reference's kite_prp
semantics); an LLR test whose V is non-zero is confirmed by a second run at the next longer FFT
and, if they disagree, a third (src/llr.c:457-534).  The verified state of every test is
checkpointed every `checkpoint_every` iterations in the reference's formats (KITECKP1,
KITELLR1).  The report gives p50/p99 time-to-verdict, tests/hour and every verdict's RES64.
"""
from __future__ import annotations

import math
import os
import time
from collections import deque
from dataclasses import dataclass, field

from . import native
from .kite import Batch

FERMAT, LLR = "fermat", "llr"


@dataclass
class Request:
    rid: int
    kind: str
    k: int
    n: int
    arrival: float          # seconds after the start of serving


@dataclass
class Verdict:
    rid: int
    kind: str
    k: int
    n: int
    res64: int
    is_prime: bool          # Fermat: PRP; LLR: prime
    arrival: float
    done: float
    fft_len: int
    maxerr: float
    squarings: int
    runs: int = 1
    rc: int = 0
    factor: int = 0         # LLR: the small factor that decided the test, else 0

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def poisson_requests(seed: int, rate_per_s: float, duration_s: float, fermat_share: float = 0.8,
                     k_range=(3, 10_000), n_range=(100_000, 4_000_000)):
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    lo, hi = math.log(n_range[0]), math.log(n_range[1])
    while True:
        t += float(rng.exponential(1.0 / rate_per_s))
        if t > duration_s:
            return out
        kind = FERMAT if rng.random() < fermat_share else LLR
        while True:  # k odd and uniform in k_range: an even upper bound's k_range[1] + 1 is redrawn
            k = int(rng.integers(k_range[0] // 2, k_range[1] // 2 + 1)) * 2 + 1
            if k <= k_range[1]:
                break
        n = int(math.exp(rng.uniform(lo, hi)))
        out.append(Request(len(out), kind, k, n, t))


def next_fft_len(L: int) -> int:
    """The next usable FFT length above L (reference src/ctx.c:143-148)."""
    m = (L // 64 + 1) * 64
    while True:
        x = m
        for p in (2, 3, 5, 7):
            while x % p == 0:
                x //= p
        if x == 1:
            return m
        m += 64


@dataclass
class _Running:
    req: Request
    run: int                        # LLR: 0 first run, 1-2 confirmations
    fft_len: int = 0
    res64s: list = field(default_factory=list)
    zeros: list = field(default_factory=list)
    squarings: int = 0
    maxerr: float = 0.0
    next_ckpt: int = 0


class Server:
    def __init__(self, gerbicz_block: int = 500, mem_budget: int = 0, checkpoint_dir: str | None = None,
                 checkpoint_every: int = 100_000, device: int = -1):
        self.batch = Batch(gerbicz_block=gerbicz_block, mem_budget=mem_budget, device=device)
        self.lib = native.load()
        self.ckdir = checkpoint_dir
        self.ck_every = checkpoint_every
        self.checkpoints = 0
        if checkpoint_dir:
            os.makedirs(checkpoint_dir, exist_ok=True)

    def close(self):
        self.batch.close()

    def _admit(self, run: _Running) -> int:
        r = run.req
        if r.kind == FERMAT:
            return self.batch.add_fermat(r.k, r.n, 3, run.fft_len)
        return self.batch.add_llr(r.k, r.n, run.fft_len)

    def serve(self, requests, max_seconds: float | None = None, clock=time.monotonic):
        """Serve the requests in arrival order, in real time; returns (verdicts, stats)."""
        pending = deque(sorted(requests, key=lambda q: q.arrival))
        waiting: deque[_Running] = deque()
        active: dict[int, _Running] = {}
        verdicts: list[Verdict] = []
        start = clock()
        blocks = 0
        peak_active = 0
        while pending or waiting or active:
            now = clock() - start
            if max_seconds is not None and now > max_seconds:
                break
            while pending and pending[0].arrival <= now:
                waiting.append(_Running(pending.popleft(), 0))
            while waiting:
                slot = self._admit(waiting[0])
                if slot == -2:          # memory budget full: wait for slots to free up
                    break
                run = waiting.popleft()
                if slot < 0:            # not a valid test for this engine
                    verdicts.append(Verdict(run.req.rid, run.req.kind, run.req.k, run.req.n, 0, False,
                                            run.req.arrival, now, 0, 0.0, 0, run.run + 1, rc=-1))
                    continue
                run.next_ckpt = self.ck_every
                active[slot] = run
            peak_active = max(peak_active, len(active))
            if not active:
                if pending:
                    time.sleep(max(0.0, min(0.05, pending[0].arrival - (clock() - start))))
                continue
            self.batch.step(1)
            blocks += 1
            done_t = clock() - start
            for slot in list(active):
                run = active[slot]
                st, res = self.batch.result(slot)
                if st == 0:
                    if self.ckdir and res.iter >= run.next_ckpt:
                        path = os.path.join(self.ckdir, f"{run.req.kind}_{run.req.rid}.ckpt")
                        if self.lib.kc_batch_checkpoint(self.batch.h, slot, path.encode()) == 0:
                            self.checkpoints += 1
                        run.next_ckpt = (res.iter // self.ck_every + 1) * self.ck_every
                    continue
                del active[slot]
                self.batch.release(slot)
                run.squarings += res.squarings
                run.maxerr = max(run.maxerr, res.maxerr)
                run.fft_len = res.fft_len
                r = run.req
                if st == 2 or res.rc != 0:
                    verdicts.append(Verdict(r.rid, r.kind, r.k, r.n, res.res64, False, r.arrival, done_t,
                                            res.fft_len, run.maxerr, run.squarings, run.run + 1, rc=res.rc or -1))
                    continue
                if r.kind == FERMAT:
                    verdicts.append(Verdict(r.rid, r.kind, r.k, r.n, res.res64, bool(res.is_prp), r.arrival,
                                            done_t, res.fft_len, run.maxerr, run.squarings))
                    continue
                # LLR: a factor or V == 0 decides at once; a non-zero V is confirmed
                if res.factor:
                    verdicts.append(Verdict(r.rid, r.kind, r.k, r.n, 0, False, r.arrival, done_t, 0, 0.0, 0,
                                            factor=int(res.factor)))
                    continue
                run.res64s.append(res.res64)
                run.zeros.append(bool(res.is_prp))
                decided = None
                if run.run == 0 and run.zeros[0]:
                    decided = 0
                elif run.run == 1 and (run.res64s[1], run.zeros[1]) == (run.res64s[0], run.zeros[0]):
                    decided = 1
                elif run.run == 2:
                    if (run.res64s[2], run.zeros[2]) == (run.res64s[1], run.zeros[1]):
                        decided = 2
                    elif (run.res64s[2], run.zeros[2]) == (run.res64s[0], run.zeros[0]):
                        decided = 0
                    else:
                        verdicts.append(Verdict(r.rid, r.kind, r.k, r.n, 0, False, r.arrival, done_t,
                                                res.fft_len, run.maxerr, run.squarings, 3, rc=-3))
                        continue
                if decided is not None:
                    verdicts.append(Verdict(r.rid, r.kind, r.k, r.n, run.res64s[decided], run.zeros[decided],
                                            r.arrival, done_t, res.fft_len, run.maxerr, run.squarings,
                                            run.run + 1))
                else:  # confirmation run at the next longer FFT, ahead of new arrivals
                    run.run += 1
                    run.fft_len = next_fft_len(res.fft_len)
                    waiting.appendleft(run)
        elapsed = clock() - start
        lat = sorted(v.latency for v in verdicts if v.rc == 0)
        stats = {
            "elapsed_s": elapsed,
            "completed": len([v for v in verdicts if v.rc == 0]),
            "failed": len([v for v in verdicts if v.rc != 0]),
            "in_flight": len(active) + len(waiting) + len(pending),
            "tests_per_hour": 3600.0 * len(lat) / elapsed if elapsed > 0 else 0.0,
            "p50_s": _percentile(lat, 50),
            "p99_s": _percentile(lat, 99),
            "blocks": blocks,
            "peak_active": peak_active,
            "checkpoints": self.checkpoints,
            "gpu_s": self.batch.gpu_ms / 1e3,
        }
        return verdicts, stats


def _percentile(sorted_vals, p):
    if not sorted_vals:
        return None
    i = min(len(sorted_vals) - 1, max(0, int(math.ceil(p / 100.0 * len(sorted_vals))) - 1))
    return sorted_vals[i]


def main():
    import argparse
    import json
    ap = argparse.ArgumentParser(description="served Fermat/LLR request loop on one GPU")
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--rate", type=float, default=2.0, help="arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="seconds of arrivals")
    ap.add_argument("--max-seconds", type=float, default=None, help="stop serving after this")
    ap.add_argument("--n-min", type=int, default=100_000)
    ap.add_argument("--n-max", type=int, default=4_000_000)
    ap.add_argument("--block", type=int, default=500)
    ap.add_argument("--checkpoint-dir", default=None)
    args = ap.parse_args()
    reqs = poisson_requests(args.seed, args.rate, args.duration, n_range=(args.n_min, args.n_max))
    srv = Server(gerbicz_block=args.block, checkpoint_dir=args.checkpoint_dir)
    try:
        verdicts, stats = srv.serve(reqs, max_seconds=args.max_seconds)
    finally:
        srv.close()
    stats["requests"] = len(reqs)
    print(json.dumps(stats))
    for v in sorted(verdicts, key=lambda v: v.rid):
        print(json.dumps({"id": v.rid, "kind": v.kind, "k": v.k, "n": v.n, "res64": f"{v.res64:016X}",
                          "prime": v.is_prime, "latency_s": round(v.latency, 3), "fft_len": v.fft_len,
                          "maxerr": round(v.maxerr, 4), "runs": v.runs, "rc": v.rc, "factor": v.factor}))


if __name__ == "__main__":
    main()
