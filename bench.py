"""Benchmark: Fermat base-3 tests per hour, batched on one GB300 (and one-at-a-time for
comparison), with the reference's CPU path timed on the host cores beside it.

Workload (the batched configuration): 256 concurrent Fermat base-3 PRP tests of N = k*2^n - 1,
k uniform odd in [3, 10^4], n uniform integer in [300000, 700000] (numpy PCG64, seed 3), each at
the FFT length the reference's length chooser picks (16K-56K words).  Synthetic, seeded: the
reference publishes no benchmark suite.

A step is one Gerbicz block of every test: B = 1000 squarings of each test's x (one CUDA graph:
the tests in three parts of about equal work, each part's 3000 pass launches on its own stream)
plus the block's product d <- d*x, and for the tests at the end of a round the check (B
squarings of t and a product instead of x's, then the comparison on the device).  The first
round of the j-th test is 1 + (j mod M) blocks (kc_batch_stagger_checks), so the checks fall on
different blocks as in a batch refilled over time, and every timed block holds the steady
state's share of them.  Throughput is measured progress: tests/hour = 3600 * (squarings of x
advanced by all tests) / (T_blocks * mean(n)).

  value     T_blocks from CUDA events around the work on the batch stream
  e2e       the same through the C ABI with host buffers: wall-clock kc_batch_step calls (their
            H2D slot tables and work lists, D2H round-off), plus per-test admission (H2D of
            x0 and the tables) and read-back (D2H of the residue), amortised per test
  roofline  a block's algorithmic FP64 FLOPs (its kernels run concurrently on three streams)
            over the block's CUDA-event time, against the FP64 FMA peak measured on this GPU
            by a DFMA kernel
  cpu_baseline  the reference's arithmetic on the host: the CPU oracle's port of the
            reference's `ref` backend (one test per core on all cores) over a bounded sample

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank runs its own independent batch (replicas; the tests do not shard).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SLOTS = 256
BLOCK = 1000
BLOCKS_PER_CHECK = 250
SEED = 3
WORKLOAD = "fermat-batch-256: k odd U[3,1e4], n U[300000,700000], base 3, B=1000, M=250"


def bench_config(lengths: dict, mean_n: float) -> dict:
    """The workload as both arms report it (the reference arm computes the same lengths)."""
    return {"workload": WORKLOAD, "slots": SLOTS, "mean_n": mean_n,
            "fft_lengths": {str(k): v for k, v in sorted(lengths.items())},
            "checks": f"Gerbicz check every M={BLOCKS_PER_CHECK} blocks, first rounds staggered by "
                      "admission order (check work inside the timed blocks)",
            "l2": "inputs larger than L2 (~256 x 0.3 MB numbers + 0.6 MB tables per test)"}


def workload(seed: int = SEED, count: int = SLOTS):
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    ks = rng.integers(1, 5000, size=count) * 2 + 1      # odd in [3, 9999]
    ns = rng.integers(300000, 700001, size=count)
    return [(int(k), int(n)) for k, n in zip(ks, ns)]


def combine_ranks(t_block: float, t_block_wall: float, per_rank_units: float, dist=None):
    """Replicas: every rank ran its own batch.  The step time is the slowest rank's (max over
    ranks) and the whole-job throughput is the sum of the ranks' units over that time, i.e.
    world x units / max time.  Returns (t_block, t_block_wall, world)."""
    world = 1
    if dist is not None and dist.is_initialized():
        import torch
        world = dist.get_world_size()
        tt = torch.tensor([t_block, t_block_wall], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_block, t_block_wall = float(tt[0]), float(tt[1])
    return t_block, t_block_wall, world


def rank_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_sample(tests, threads: int, squarings: int):
    """The oracle (a port of the reference's ref backend) on `threads` host cores: one test per
    core, `squarings` squarings each; returns (tests/hour, seconds of CPU work, detail)."""
    from oracle import oracle
    oracle.build(ref=False)
    sample = [(k, n, oracle.choose_fft_len(k, n)) for k, n in tests]
    t0 = time.perf_counter()
    us = oracle.time_squarings(sample, threads, squarings)
    wall = time.perf_counter() - t0
    per_test_s = [n * u * 1e-6 * (1 + 1 / BLOCKS_PER_CHECK + 2 / BLOCK) for (k, n, _), u in zip(sample, us)]
    tph = threads * 3600.0 / statistics.mean(per_test_s)
    return tph, wall * threads, {"tests": len(sample), "squarings_each": squarings,
                                 "us_per_sq_mean": statistics.mean(us)}


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build(ref=False)
    threads = os.cpu_count() or 1
    tests = workload()
    mean_n = statistics.mean(n for _, n in tests)
    lengths = {}
    for k, n in tests:
        L = oracle.choose_fft_len(k, n)
        lengths[L] = lengths.get(L, 0) + 1
    sample = tests[:threads]
    squarings = 64
    # each step: one test per core, a bounded number of squarings each
    for _ in range(args.warmup):
        cpu_sample(sample, threads, 4)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tph, work, det = cpu_sample(sample, threads, squarings)
        vals.append(tph)
    wall = time.perf_counter() - t0
    value = statistics.median(vals)
    desc = (f"{len(sample)} of the 256 tests (one per core) x {squarings} squarings per step, "
            "extrapolated to full tests (n squarings, Gerbicz overhead 1/M + 2/B)")
    line = {
        "impl": "reference", "metric": "fermat_tests_per_hour", "value": value,
        "unit": "tests/hour", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
        "config": bench_config(lengths, mean_n),
        "cpu_baseline": {"value": value, "unit": "tests/hour", "cores": threads, "kind": "port",
                         "sample": desc, "note": PORT_NOTE},
        "e2e": {"value": value, "unit": "tests/hour", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# The reference's own `ref` backend cannot be built on the GPU host (its sources stay in the build
# container and binaries built there do not run on the Arm host), so the CPU figure is the
# oracle's port of it.  Measured single-threaded in the build container (oracle/_ref built from
# the reference sources): ref 8.15 / 10.2 / 17.3 ms per squaring at L = 28672 / 36864 / 49152,
# the port 2.03 / 2.31 / 3.01 ms: the port is 4.0-5.8x faster, so this baseline favours the CPU.
PORT_NOTE = ("the oracle's port of the reference's ref backend; in the build container the port "
             "was 4.0-5.8x faster per squaring than the reference's own ref build (L 28672-49152)")


# parts (streams) of a block's pass launches (the batch's default, KITE_GB300_BATCH_SPLIT)
PARTS = 3
# squarings of every test per launch of the persistent kernel, timed beside the block for
# comparison (the batch's default KITE_GB300_STEPS_PER_LAUNCH)
STEPS_PER_LAUNCH = 100
# Per squaring of this workload's 256 tests in the block's form, from one ncu capture of the nine
# pass launches of one squaring (three parts of three passes; ncu serialises them):
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,sm__sass_thread_inst_executed_op_
#   {dfma,dadd,dmul}_pred_on.sum,... --clock-control none -k 'regex:k_rows|k_col_inverse|k_col_forward'
#   -s 256 -c 9 python bench.py --quick --steps 1 --warmup 1 --no-ntt
# (the 256 launches skipped are the tests' admission).  A block is B + 1 squaring-sized passes.
# DRAM: 421.9 MB read + 11.2 MB written (ncu runs the three parts one after another; concurrent,
# the persistent form of the same passes moved 556 MB per squaring).  FP64 lane operations: 479.0e6
# per squaring on average, from a 100-squaring capture of the same item functions (the single
# squaring above, 499.9e6, is a step that also tracks round-off, which one step in four does).
K_SQ_DRAM_BYTES = 433.1e6
K_SQ_FP64_LANE_OPS = 479.0e6
K_SQ_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the nine pass launches of one "
                       "squaring, times B + 1 (profiles/launches_fermat_batch256.md)")


def run_ours(args):
    rank, world, local = rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("gloo")
    from ahnum_gb300.build import build_library
    build_library()
    from ahnum_gb300 import native
    from ahnum_gb300.kite import Batch, Ctx
    lib = native.load()
    device = local
    import ctypes as C

    # the autotuned four-step shapes of this GPU, batched and single-test (shapes only: the FFT
    # lengths stay the ones the reference's length chooser picks)
    from ahnum_gb300.tune import load_gb300_tuning
    load_gb300_tuning(lib)

    tests = workload(seed=SEED + rank)
    mean_n = statistics.mean(n for _, n in tests)

    # ---- admission (H2D of x0 digits and tables), timed for e2e
    b = Batch(gerbicz_block=BLOCK, gerbicz_blocks=BLOCKS_PER_CHECK, device=device)
    lib.kc_batch_stagger_checks(b.h, 1)
    t0 = time.perf_counter()
    slots = [b.add_fermat(k, n) for k, n in tests]
    t_admit = time.perf_counter() - t0
    assert all(s >= 0 for s in slots), "admission failed"
    lengths = {}
    for s in slots:
        st, r = b.result(s)
        lengths[r.fft_len] = lengths.get(r.fft_len, 0) + 1

    # ---- warm-up blocks (graph capture, clocks)
    for _ in range(args.warmup):
        b.step(1)

    def positions():
        return [b.result(s)[1].position for s in slots]

    # ---- timed region: K blocks, events on the batch stream, barrier + max over ranks
    before = positions()
    if dist:
        dist.barrier()
    gpu_ms = []
    wall = []
    with Clocks(device) as clk:
        for _ in range(args.steps):
            ms = C.c_double()
            w0 = time.perf_counter()
            r = lib.kc_batch_step(b.h, 1, C.byref(ms))
            wall.append(time.perf_counter() - w0)
            if r < 0:
                raise RuntimeError(f"kc_batch_step failed {r}")
            gpu_ms.append(ms.value)
    if dist:
        dist.barrier()
    progress = sum(a - p for a, p in zip(positions(), before))  # squarings of x advanced
    check_blocks = (SLOTS * BLOCK * args.steps - progress) / BLOCK
    t_block, t_block_wall, _ = combine_ranks(statistics.mean(gpu_ms) * 1e-3, statistics.mean(wall),
                                             SLOTS, dist)

    per_rank = 3600.0 * progress / (t_block * args.steps * mean_n)
    value = per_rank * world

    h2d = C.c_uint64()
    d2h = C.c_uint64()
    lib.kc_batch_last_transfer(b.h, C.byref(h2d), C.byref(d2h))

    # largest round-off of every slot over its blocks so far (warm-up and timed), against the
    # drivers' 0.40 limit; a slot above it would have been restarted at a longer FFT
    roundoff = {"max": 0.0, "limit": 0.40, "retries": 0, "gerbicz_errors": 0,
                "over": f"{args.warmup + args.steps} blocks of every test (warm-up and timed)"}
    for s in slots:
        st, r = b.result(s)
        roundoff["max"] = max(roundoff["max"], r.maxerr)
        roundoff["retries"] += r.roundoff_retries
        roundoff["gerbicz_errors"] += r.gerbicz_errors

    # ---- read-back of every residue (D2H + exact host conversion), timed for e2e
    t0 = time.perf_counter()
    for (k, n), s in zip(tests, slots):
        limbs = (C.c_uint64 * ((n + 127) // 64))()
        if lib.kc_batch_read(b.h, s, limbs) != 0:
            raise RuntimeError("kc_batch_read failed")
    t_read = time.perf_counter() - t0
    e2e_per_test = (t_admit + t_read) / SLOTS + mean_n * t_block_wall * args.steps / progress
    e2e_value = 3600.0 / e2e_per_test * world

    # ---- roofline (after the timed region): the block's algorithmic FLOPs over its CUDA-event
    #      time (its kernels overlap on three streams); each pass alone and the persistent kernel,
    #      on the batch stream, for the split of the time and for comparison
    ms3 = (C.c_double * 3)()
    fl3 = (C.c_double * 3)()
    lib.kc_batch_profile(b.h, 5, ms3, fl3)
    msp, flp = C.c_double(), C.c_double()
    if lib.kc_batch_profile_steps(b.h, STEPS_PER_LAUNCH, C.byref(msp), C.byref(flp)) != 0:
        raise RuntimeError("kc_batch_profile_steps failed")
    peak = lib.kc_fp64_peak(device)
    flops_sq = fl3[0] + fl3[1] + fl3[2]          # one squaring of every test
    flops_block = flops_sq * (BLOCK + 1)          # B squarings and the product
    achieved = flops_block / t_block
    names = ["k_rows (row FFT + split square), alone", "k_col_inverse (inverse column FFT + round + carry), alone",
             "k_col_forward (carry-in + forward column FFT), alone"]
    kernels = {names[q]: {"ms_per_launch": ms3[q], "gflop_per_launch": fl3[q] / 1e9,
                          "tflops": fl3[q] / (ms3[q] * 1e-3) / 1e12 if ms3[q] else 0}
               for q in range(3)}
    kernels[f"k_squarings (persistent form, {STEPS_PER_LAUNCH} squarings of every test per launch)"] = {
        "ms_per_launch": msp.value, "gflop_per_launch": flp.value / 1e9,
        "tflops": flp.value / (msp.value * 1e-3) / 1e12 if msp.value else 0}
    b.close()

    ntt = ntt_leg(lib, tests, mean_n, device) if args.ntt else None

    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": "fermat_tests_per_hour", "value": value, "unit": "tests/hour",
                              "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": t_block * 1e3, "quick": True, "kernels": kernels,
                              "roundoff": roundoff,
                              "ntt_engine": ntt}), flush=True)
        if dist:
            dist.destroy_process_group()
        return

    # ---- single-test GPU path on the same tests (one at a time), per distinct length
    single = {}
    for L in sorted(lengths):
        k, n = next((k, n) for k, n in tests if _len(lib, k, n) == L)
        with Ctx(k, n) as c:
            x = c.num(3)
            c.square(x, 20)
            c.sync()
            s0 = time.perf_counter()
            c.square(x, 200)
            c.sync()
            single[L] = (time.perf_counter() - s0) / 200
    single_s = [n * single[_len(lib, k, n)] * (1 + 1 / BLOCKS_PER_CHECK + 2 / BLOCK) for k, n in tests]
    single_tph = 3600.0 / statistics.mean(single_s)
    with Ctx(9001, 662695, 49152) as c:
        x = c.num(3)
        c.square(x, 50)
        c.sync()
        s0 = time.perf_counter()
        c.square(x, 1000)
        c.sync()
        us_sq_49152 = (time.perf_counter() - s0) / 1000 * 1e6

    large = large_segment(lib) if rank == 0 else None

    cpu = None
    if rank == 0:
        threads = os.cpu_count() or 1
        tph, work, det = cpu_sample(tests[:threads], threads, args.cpu_squarings)
        cpu = {"value": tph, "unit": "tests/hour", "cores": threads, "kind": "port",
               "sample": f"{det['tests']} of the 256 tests, one per core, {det['squarings_each']} "
                         f"squarings each ({work:.1f} s of CPU work), extrapolated to full tests",
               "note": PORT_NOTE}

    if rank == 0:
        line = {
            "metric": "fermat_tests_per_hour", "value": value, "unit": "tests/hour",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_block * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
            "config": bench_config(lengths, mean_n),
            "timed_progress": {"squarings_of_x": progress, "check_blocks": check_blocks,
                               "blocks": args.steps},
            "e2e": {"value": e2e_value, "unit": "tests/hour", "h2d_bytes_per_step": h2d.value,
                    "d2h_bytes_per_step": d2h.value,
                    "admission_s": t_admit, "readback_s": t_read, "block_wall_s": t_block_wall},
            "roundoff": roundoff,
            # per block: the three passes of each part, the block's product (three passes), and
            # per check block two digit passes and the comparison kernel
            "gpu_launches": int(args.steps * (PARTS * 3 * BLOCK + 3) + 3 * check_blocks),
            "clocks": clk.summary(),
            "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12,
                         "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                         "traffic": K_SQ_DRAM_BYTES * (BLOCK + 1) if K_SQ_DRAM_BYTES else None,
                         "traffic_source": K_SQ_TRAFFIC_SOURCE,
                         # FP64 instructions actually issued (ncu count) against the probe's
                         # instruction rate (peak / 2: the probe's DFMAs count 2 FLOPs each)
                         "fp64_issue": None if not K_SQ_FP64_LANE_OPS else {
                             "lane_ops_per_block": K_SQ_FP64_LANE_OPS * (BLOCK + 1),
                             "per_second": K_SQ_FP64_LANE_OPS * (BLOCK + 1) / t_block,
                             "vs_probe_rate": K_SQ_FP64_LANE_OPS * (BLOCK + 1) / t_block / (peak / 2) if peak else None},
                         "kernel": f"one Gerbicz block: the pass kernels of {BLOCK} squarings in {PARTS} parts on "
                                   f"{PARTS} streams, and the product (one CUDA graph; the unit is the block)",
                         "peak_source": "measured: DFMA dependent-chain kernel on this GPU "
                                        "(MEASURED_PEAKS.json has no FP64 figure)"},
            "kernels": kernels,
            "single_test": {"tests_per_hour": single_tph, "us_per_squaring_L49152": us_sq_49152,
                            "us_per_squaring_by_L": {str(L): v * 1e6 for L, v in sorted(single.items())},
                            "batched_over_single": value / world / single_tph},
            "cpu_baseline": cpu,
            "large_single_test": large,
            "ntt_engine": ntt,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def large_segment(lib, seed=4, squarings=100_000, block=1000, blocks_per_check=50):
    """The large single test: a Fermat test of k*2^n-1, k odd seeded in [3, 255], n seeded in
    [2e7, 2.5e7] (FFT length about 1.2-1.8 M words), stopped after `squarings` verified
    squarings.  Gerbicz blocks of 1000 with a check every 50 blocks, so the segment holds two
    checks.  Time per squaring from the progress callbacks (one per block, after a device sync),
    checks included."""
    import ctypes as C
    import numpy as np
    from ahnum_gb300 import native
    rng = np.random.Generator(np.random.PCG64(seed))
    k = int(rng.integers(1, 128)) * 2 + 1
    n = int(rng.integers(20_000_000, 25_000_001))
    flag = C.c_int(0)
    marks = []

    def progress(arg, it, nn, e):
        marks.append((time.perf_counter(), int(it), float(e)))
        if it >= squarings:
            flag.value = 1

    cb = native.PROGRESS_FN(progress)
    o = native.KitePrpOpts()
    o.fft = native.KiteOpts(native.KITE_BACKEND_CUDA, 0, 0, 0)
    o.gerbicz_block = block
    o.gerbicz_blocks = blocks_per_check
    o.progress = cb
    o.abort_flag = C.pointer(flag)
    r = native.KitePrpResult()
    t0 = time.perf_counter()
    rc = lib.kite_prp(k, n, 3, C.byref(o), C.byref(r))
    wall = time.perf_counter() - t0
    (ta, ia, _), (tb, ib, _) = marks[0], marks[-1]
    return {"k": k, "n": n, "fft_len": lib.kc_choose_fft_len(k, n), "squarings": ib,
            "us_per_squaring": (tb - ta) / (ib - ia) * 1e6, "wall_s": wall,
            "gerbicz_block": block, "gerbicz_blocks_per_check": blocks_per_check,
            "gerbicz_errors": r.gerbicz_errors, "maxerr": max(e for _, _, e in marks),
            "stopped_on_request": rc == -5}


def ntt_leg(lib, tests, mean_n, device, blocks=3):
    """The same tests on the exact integer-NTT engine (include/kite_ntt.h): a lockstep Gerbicz
    batch (ahnum_gb300.ntt_group.NttFermatBatch) of all tests, B = 1000, M = 250, timed over
    `blocks` blocks of B squarings and the block product (CUDA events on the groups' streams);
    tests/hour with the FP64 line's block accounting."""
    from ahnum_gb300.ntt_group import NttFermatBatch, time_steps
    with NttFermatBatch(tests, block=BLOCK, blocks_per_check=BLOCKS_PER_CHECK, device=device) as nb:
        nb.run(max_blocks=1)  # graphs, clocks
        nb.block_ms, nb.blocks = 0.0, 0
        nb.run(max_blocks=blocks)
        t_block = nb.block_ms * 1e-3 / nb.blocks
    t_sq, nps = time_steps(tests, 64, 3, device)
    tph = 3600.0 * len(tests) * BLOCK / (t_block * (1 + 1 / BLOCKS_PER_CHECK) * mean_n)
    return {"tests_per_hour": tph, "ms_per_block": t_block * 1e3, "ms_per_squaring_step": t_sq * 1e3,
            "us_per_test_squaring": t_sq * 1e6 / len(tests),
            "transform_lengths": {str(k): v for k, v in nps.items()},
            "gpu_launches_per_squaring": 4,
            "arithmetic": "exact: residues mod three or four 30-bit primes, Garner CRT, Montgomery R=2^n"}


_len_cache = {}


def _len(lib, k, n):
    key = (k, n)
    if key not in _len_cache:
        _len_cache[key] = lib.kc_choose_fft_len(k, n)
    return _len_cache[key]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-squarings", type=int, default=300)
    ap.add_argument("--no-ntt", dest="ntt", action="store_false",
                    help="skip the integer-NTT engine's line on the same tests")
    ap.add_argument("--quick", action="store_true",
                    help="skip the single-test and CPU legs (for profiler runs)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
