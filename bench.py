#!/usr/bin/env python3
"""Benchmark of the GB300 dense Goldbach verify path.

Headline workload: production segments of 467.5M integers at 4e18 + k *
467.5e6, k drawn from seed 1 in [0, 1e5) (the reference's production
segment shape). A step is one batch of consecutive segments (128, the
committed autotuner record's choice; --batch with --tuning none): one sieve
pass over one HBM-resident class map of 2.0 GB, then per segment the
checker, prime / twin / gap statistics and the class-map hash, replayed as
the slot's captured CUDA graph. Successive steps take successive batches,
so no step repeats work, and a step's map and sieving primes (393 MB)
exceed L2.

Statistics mode (--sample-every, default 256): the reference's production
mode -- every 256th segment of the run gets p(n) of every even (its
GB_STATS_SAMPLE default), the others the funnel verify plus the exact p(n)
of every even the plan leaves (which holds every even with p(n) >= 3000);
primes, twins and the full gap walk on every segment. `exact_all` repeats
the measurement with p(n) of every even on every segment.

value  = evens verified per second over the timed steps, device time from
         CUDA events recorded on the launching stream around every stage
         (inputs resident in HBM).
e2e    = the same metric through the C ABI as a caller uses it: two slots in
         flight, gbc_enqueue_batch + gbc_collect, per-segment results copied
         to host memory inside the timed region, wall clock.
plain  = the plain form on the same GPU, as the reference runs it: the hit
         lists harvested once per batch of segments, then every segment
         through its own launches of the sieve, large-prime, checker and
         count kernels (launch mode 3); batched_over_plain is value /
         plain.value (device) and e2e / plain.e2e. plain_one_segment_batches:
         one segment per batch with every stage, the hit lists included, per
         segment.
windows = 256 windows of log-uniform widths in [1e6, 1e10] at uniform starts
         in [1e15, 5e18] (seed 7) verified in shared batches, against the same
         windows run one at a time; every window's statistics compared.
serving = Poisson arrivals at 50 windows/s for 60 s (seed 11), widths
         log-uniform in [1e4, 1e9], starts log-uniform in [1e10, 5e18], served
         by the continuous-batching loop under a 150 GB HBM budget: p50 / p99
         latency from submission to completion, sustained evens/s, and a
         sample of windows compared with their runs alone.
sparse = the sparse class map cross-check (12 residue classes mod 30030,
         candidates to 4e7): --sparse-segments full segments of 30030 *
         2^--sparse-dlt-log2 integers from 4e18, a warm pass then a timed
         one; value from CUDA events, e2e the wall time of the call.
         --sparse-only runs this leg alone.
--slice runs the full 5e13-wide slice at 4e18 batched and plain, and checks
3 seeded segments against the CPU oracle.
--impl reference times the reference's CPU algorithm (the oracle's
restatement of tests/stats_ref.cpp: Miller-Rabin p(n) of every even, run on
every host core) on a bounded sample of the same workload.
"""
import argparse
import ctypes
import json
import os
import random
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "goldbach-l0_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

SEG = 467_500_000
METRIC = "G evens/s at 4e18, bit-exact stats: batched vs plain on 1 GB300; p99 latency"
NPRIMES_4E18 = 98_222_287   # odd primes <= 2.0e9 = sqrt of the workload's end


def workload_start():
    k = random.Random(1).randrange(100000)
    return 4 * 10**18 + k * SEG


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_counters():
    """kernel -> (DRAM bytes, warp instructions or None) per launch from
    profiles/ncu_counters.txt (lines "kernel dram_bytes warp_inst note";
    "-" for instructions not measured at this size)."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_counters.txt")) as f:
            for ln in f:
                t = ln.split()
                if len(t) >= 3 and not ln.startswith("#"):
                    out[t[0]] = (float(t[1]), None if t[2] == "-" else float(t[2]))
    except OSError:
        pass
    return out


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index=None):
        self.rows, self.proc = [], None
        self.index = str(index) if index is not None else os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,clocks.mem,"
                 "temperature.gpu",
                 "--format=csv,noheader,nounits", "-i", self.index,
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.rows.append([x.strip() for x in ln.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        mem = [float(r[8]) for r in self.rows if len(r) > 8 and r[8].replace(".", "").isdigit()]
        temp = [float(r[9]) for r in self.rows if len(r) > 9 and r[9].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "mem_mhz": statistics.median(mem) if mem else None, "temp_c": max(temp) if temp else None,
                "reasons": reasons, "samples": len(self.rows)}


class Replicas:
    """N independent replicas (python -m torch.distributed.run ...
    bench.py --gpus N): rank r verifies its own consecutive segments on GPU
    LOCAL_RANK. The path shards by segment with no exchange, so the only
    communication is host-side: a barrier on both sides of the timed
    region and the max over ranks of the time (gloo)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist and self.dist.is_initialized():
            self.dist.destroy_process_group()


def batches(start, first_seg, nbatch, batch):
    """nbatch batches of `batch` segments from segment index first_seg."""
    out = []
    for b in range(nbatch):
        segs = []
        for j in range(batch):
            i = first_seg + b * batch + j
            s = start + i * SEG
            segs.append((i, s, s + SEG - 2))
        out.append(segs)
    return out


def seg_args(b, sample_every, gbc):
    return [(s, e) for _, s, e in b], [0 if sample_every <= 1 or i % sample_every == 0 else gbc.SEG_VERIFY
                                       for i, _, _ in b]


def cpu_baseline(evens, start):
    import oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.stats_line(start, start + 2 * (evens - 1), oracle.MR, threads)
    dt = time.perf_counter() - t0
    return {"value": evens / dt / 1e9, "unit": "G evens/s", "cores": threads, "kind": "port",
            "sample": f"{evens} evens from {start}: the oracle's restatement of tests/stats_ref.cpp "
                      f"(Miller-Rabin p(n) of every even, primes, twins, gaps) on {threads} threads, {dt:.2f} s"}


def run_reference(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    start = workload_start()
    per_step = args.ref_evens
    for i in range(args.warmup):
        cpu_baseline(per_step // 10, start + 2 * per_step * i)
    t0 = time.perf_counter()
    for i in range(args.steps):
        cpu_baseline(per_step, start + 2 * per_step * (args.warmup + i))
    dt = time.perf_counter() - t0
    v = per_step * args.steps / dt / 1e9
    cores = os.cpu_count() or 1
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "G evens/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": f"{per_step} evens per step of the production segments at {start}",
                       "segment": SEG},
            "cpu_baseline": {"value": v, "unit": "G evens/s", "cores": cores, "kind": "port",
                             "sample": f"{per_step} evens per step, Miller-Rabin per even (tests/stats_ref.cpp's "
                                       f"algorithm, restated in oracle/gb_oracle.c), {cores} threads"},
            "e2e": {"value": v, "unit": "G evens/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def device_run(ctx, bs, limit, sample_every, gbc):
    """Steps back to back on one slot; per-stage device time from the ABI's
    CUDA events on the launching stream."""
    stage = {"tile": 0.0, "large": 0.0, "check": 0.0, "count": 0.0}
    total = 0.0
    for b in bs:
        segs, flags = seg_args(b, sample_every, gbc)
        ctx.enqueue_batch(0, segs, limit, flags)
        _, t = ctx.collect(0, len(segs))
        total += t.ms_total
        stage["tile"] += t.ms_tile
        stage["large"] += t.ms_large
        stage["check"] += t.ms_check
        stage["count"] += t.ms_count
    return total, stage


def plain_leg(gbc, start, nseg, first_seg, knobs=None):
    """The plain per-segment form: batches of one segment, kernels launched
    one by one (no graph), the prime-multiplier table built once before
    timing. value: device time of nseg segments back to back on one slot
    (CUDA events, as the batched value); e2e: wall time of the next nseg
    segments with two slots in flight, the reference's double-buffered
    loop."""
    segs = [(start + i * SEG, start + i * SEG + SEG - 2) for i in range(first_seg, first_seg + 2 * nseg + 1)]
    limit = segs[-1][1]
    k = {n: v for n, v in (knobs or {}).items()
         if n in ("p_mid", "mtab_max_gb", "tile_log2", "plan_funnels", "verify_funnels")}
    with gbc.Context(limit=limit, segment_even=SEG, max_batch=1, launch_mode=2, hl_mode=1, **k) as ctx:
        for sl in (0, 1):                                     # warm-up: tables, both slots
            ctx.enqueue_batch(sl, [segs[0]], limit, [gbc.SEG_VERIFY])
            ctx.collect(sl, 1)
        dev_ms = 0.0
        for s in segs[1:1 + nseg]:
            ctx.enqueue_batch(0, [s], limit, [gbc.SEG_VERIFY])
            _, t = ctx.collect(0, 1)
            dev_ms += t.ms_total
        todo = segs[1 + nseg:]
        t0 = time.perf_counter()
        for i in range(min(2, nseg)):
            ctx.enqueue_batch(i, [todo[i]], limit, [gbc.SEG_VERIFY])
        for i in range(nseg):
            ctx.collect(i & 1, 1)
            if i + 2 < nseg:
                ctx.enqueue_batch(i & 1, [todo[i + 2]], limit, [gbc.SEG_VERIFY])
        wall = time.perf_counter() - t0
    evens = nseg * (SEG // 2)
    return {"value": evens / (dev_ms / 1e3) / 1e9, "unit": "G evens/s",
            "e2e": {"value": evens / wall / 1e9, "unit": "G evens/s"}, "segments": nseg,
            "config": "one production segment per batch, kernels launched one by one, funnel verify + exact tail, "
                      "hit lists on (table built before timing), the batched form's other knobs; value: one slot, "
                      "device events; e2e: two slots in flight, wall clock"}


def plain_form_leg(gbc, start, first_seg, knobs=None, k=128):
    """The reference's plain form (src/verifier.cpp:2487-2517, 1136-1143):
    the hit lists harvested once per batch of k segments, then every segment
    through its own launches of the sieve, the large primes, the checkers and
    the count kernel (launch mode 3), production sampling. value: device time
    of one batch of k segments on one slot (CUDA events); e2e: wall time of
    the next two batches with two slots in flight."""
    segs = [(start + i * SEG, start + i * SEG + SEG - 2) for i in range(first_seg, first_seg + 4 * k)]
    limit = segs[-1][1]
    kn = {n: v for n, v in (knobs or {}).items()
          if n in ("p_mid", "mtab_max_gb", "tile_log2", "tile_bits", "plan_funnels", "verify_funnels")}
    flags = [0 if i % 256 == 0 else gbc.SEG_VERIFY for i in range(k)]
    batches = [segs[i * k:(i + 1) * k] for i in range(4)]
    with gbc.Context(limit=limit, segment_even=SEG, max_batch=k, launch_mode=3, hl_mode=1, **kn) as ctx:
        ctx.enqueue_batch(0, batches[0], limit, flags)        # warm-up: tables
        ctx.collect(0, k)
        ctx.enqueue_batch(0, batches[1], limit, flags)
        _, t = ctx.collect(0, k)
        dev_ms = t.ms_total
        t0 = time.perf_counter()
        ctx.enqueue_batch(0, batches[2], limit, flags)
        ctx.enqueue_batch(1, batches[3], limit, flags)
        ctx.collect(0, k)
        ctx.collect(1, k)
        wall = time.perf_counter() - t0
    evens = k * (SEG // 2)
    return {"value": evens / (dev_ms / 1e3) / 1e9, "unit": "G evens/s",
            "e2e": {"value": 2 * evens / wall / 1e9, "unit": "G evens/s"}, "segments_per_batch": k,
            "config": f"the plain form: hit lists harvested once per {k} segments, then each production segment "
                      "by its own launches (sieve, large primes, checkers, counts), production sampling, the "
                      "batched form's other knobs; value: one batch on one slot, device events; e2e: two batches "
                      "on two slots, wall clock"}


def log_uniform(rnd, lo, hi):
    import math
    return math.exp(rnd.uniform(math.log(lo), math.log(hi)))


def sieve_knobs(knobs):
    """The sieve knobs of a knob set (tile size, split, table budget, verify
    plan), without its batch shape."""
    keep = ("tile_log2", "tile_bits", "p_mid", "mtab_max_gb", "plan_funnels", "verify_funnels")
    return {k: v for k, v in (knobs or {}).items() if k in keep and v}


def windows_leg(gbc, n=256, seed=7, knobs=None, sample_every=0):
    """Batched uneven windows against the same windows one at a time; knobs:
    the sieve knobs of the tuning record, batches of up to 64 segments in up
    to 64 runs (16 per batch: 238 against 255 G evens/s, device time);
    sample_every 0: p(n) of every even (the campaign statistics' sampling
    of a window's first segment), gbc.SAMPLE_NONE: the funnel verify + exact
    tail everywhere (largest p(n), prime / twin counts, gaps)."""
    rnd = random.Random(seed)
    wins = []
    for _ in range(n):
        w = int(log_uniform(rnd, 1e6, 1e10)) // 2 * 2
        a = int(rnd.uniform(1e15, 5e18)) // 2 * 2
        wins.append((a, a + w))
    limit = max(b for _, b in wins)
    evens = sum((b - a) // 2 + 1 for a, b in wins)
    with gbc.Context(limit=limit, segment_even=SEG, max_batch=64, max_runs=64, nslots=3, sample_every=sample_every,
                     **sieve_knobs(knobs)) as ctx:
        ctx.prepare(min(a for a, _ in wins), limit)
        ctx.verify_windows(wins[:4])                               # warm-up: graphs
        t0 = time.perf_counter()
        out, summ = ctx.verify_windows(wins)
        wall = time.perf_counter() - t0
        t0 = time.perf_counter()
        alone = [ctx.verify_range(a, b)[1] for a, b in wins]
        wall_alone = time.perf_counter() - t0
        same = sum(1 for (_, line), al in zip(out, alone) if line == al)
        st = ctx.stats()
    return {"value": evens / wall / 1e9, "unit": "G evens/s", "windows": n, "evens": evens,
            "batches": summ.batches, "segments": summ.segments, "runs": summ.runs, "wall_s": wall,
            "alone": {"value": evens / wall_alone / 1e9, "wall_s": wall_alone},
            "batched_over_alone": wall_alone / wall, "bit_exact_vs_alone": f"{same}/{n}",
            "mtab_gb": st.mtab_bytes / 1e9,
            "config": f"{n} windows, widths log-uniform [1e6, 1e10], starts uniform [1e15, 5e18], seed {seed}, "
                      + ("funnel verify + exact tail (largest p(n), counts, gaps)" if sample_every == gbc.SAMPLE_NONE
                         else "p(n) of every even") + ", 64 segments / 64 runs per batch, 3 slots"}


def serving_leg(gbc, seconds=60.0, rate=50.0, seed=11, check=64, knobs=None):
    """Poisson arrivals into the serving loop; latency = submission to
    completion of each window."""
    rnd = random.Random(seed)
    reqs, t = [], 0.0
    while True:
        t += rnd.expovariate(rate)
        if t > seconds:
            break
        w = int(log_uniform(rnd, 1e4, 1e9)) // 2 * 2
        a = int(log_uniform(rnd, 1e10, 5e18)) // 2 * 2
        reqs.append((t, a, a + max(w, 2)))
    limit = max(b for _, _, b in reqs)
    evens = sum((b - a) // 2 + 1 for _, a, b in reqs)
    with gbc.Context(limit=limit, segment_even=SEG, max_batch=16, max_runs=16, nslots=4, **sieve_knobs(knobs)) as ctx:
        with gbc.Server(ctx, hbm_budget=150 * 10**9, lo=10**10, hi=limit) as srv:
            warm = [srv.submit(a, b) for _, a, b in reqs[:16]]      # warm-up: graphs of every slot
            for tk in warm:
                srv.wait(tk)
            tickets = [None] * len(reqs)

            def feeder():
                t0 = time.perf_counter()
                for i, (ta, a, b) in enumerate(reqs):
                    d = ta - (time.perf_counter() - t0)
                    if d > 0:
                        time.sleep(d)
                    tickets[i] = srv.submit(a, b)

            th = threading.Thread(target=feeder)
            t0 = time.perf_counter()
            th.start()
            lat, lines = [], []
            for i in range(len(reqs)):
                while tickets[i] is None:
                    time.sleep(0.0005)
                _, line, ms = srv.wait(tickets[i])
                lat.append(ms)
                lines.append(line)
            wall = time.perf_counter() - t0
            th.join()
            st = srv.stats()
        pick = random.Random(seed + 1).sample(range(len(reqs)), min(check, len(reqs)))
        same = sum(1 for i in pick if ctx.verify_range(reqs[i][1], reqs[i][2])[1] == lines[i])
    lat.sort()

    def q(x):
        return lat[min(len(lat) - 1, int(x * len(lat)))]
    return {"p50_ms": q(0.50), "p99_ms": q(0.99), "max_ms": lat[-1], "mean_ms": sum(lat) / len(lat),
            "requests": len(reqs), "rate_per_s": rate, "seconds": seconds, "evens": evens,
            "sustained": {"value": evens / wall / 1e9, "unit": "G evens/s"},
            "batches": st.batches, "segments": st.segments, "runs": st.runs,
            "max_batches_in_flight": st.max_in_flight, "gpu_busy_s": st.gpu_seconds,
            "device_gb": st.device_bytes / 1e9, "hbm_budget_gb": st.hbm_budget / 1e9,
            "bit_exact_vs_alone": f"{same}/{len(pick)}",
            "config": f"Poisson {rate}/s for {seconds} s (seed {seed}), widths log-uniform [1e4, 1e9], starts "
                      f"log-uniform [1e10, 5e18], p(n) of every even, 4 slots, 16 segments / 16 runs per batch, "
                      f"latency from submission to the window's merged statistics"}


def sparse_leg(gbc, nseg=2, dlt_log2=26):
    """The sparse class map cross-check (the reference's --sparse path):
    nseg full segments of M 2^dlt_log2 integers from 4e18 (rounded down to a
    multiple of M), one warm pass, then one timed pass; value from the
    stages' CUDA events, e2e the wall time of gbc_sparse_verify (map, checker,
    CPU resolution of the evens the GPU left)."""
    a = 4 * 10**18 - 4 * 10**18 % 30030
    span = 30030 * (1 << dlt_log2) * nseg
    t0 = time.perf_counter()
    with gbc.Sparse(limit=a + span + 10**9, dlt_log2=dlt_log2) as sp:
        init_s = time.perf_counter() - t0
        sp.verify(a, a + span - 2)
        r = sp.verify(a, a + span - 2)
    gpu_ms = r.ms_sieve + r.ms_large + r.ms_check
    return {"metric": "sparse cross-check evens verified per second", "value": r.evens / gpu_ms / 1e6,
            "unit": "G evens/s",
            "e2e": {"value": r.evens / r.ms_total / 1e6, "unit": "G evens/s", "h2d_bytes_per_step": 16,
                    "d2h_bytes_per_step": 32 * r.segments + 16 * r.pending},
            "evens": r.evens, "segments": r.segments, "pending": r.pending, "map_primes": r.map_primes,
            "entries_per_warp_task": r.groups / (r.evens / 4096), "init_s": init_s,
            "stage_ms": {"sieve": r.ms_sieve, "large": r.ms_large, "check": r.ms_check, "wall": r.ms_total},
            "config": {"workload": f"[{a}, {a + span - 2}]", "M": 30030, "K": 12, "pmax": 40_000_000,
                       "evens_per_class_per_segment": 1 << dlt_log2}}


def slice_mode(args):
    """The full 5e13 slice at 4e18, batched and plain, 3 seeded segments
    against the CPU oracle."""
    import gbc
    import oracle
    a = 4 * 10**18
    b = a + 5 * 10**13
    segs = gbc.segments_of(a, b, SEG)
    evens = (b - a) // 2 + 1
    import autotune
    knobs = autotune.load(args.tuning or autotune.DEFAULT_RECORD) if args.tuning != "none" else None
    knobs = knobs or {"max_batch": args.batch or 16}
    args.batch = knobs["max_batch"]
    with gbc.Context(limit=b, segment_even=SEG, sample_every=args.sample_every, **knobs) as ctx:
        ctx.prepare(a, b)
        res, line, _ = ctx.verify_range(a, b)
        st = ctx.stats()
    plain = plain_leg(gbc, a, args.plain_segments, 0, knobs)
    pick = sorted(random.Random(3).sample(range(len(segs)), 3))
    checks = []
    with gbc.Context(limit=b, segment_even=SEG, max_batch=1) as ctx:
        for i in pick:
            s, e = segs[i]
            t0 = time.perf_counter()
            got = ctx.verify_range(s, e)[1]
            t1 = time.perf_counter()
            want = oracle.stats_line(s, e, oracle.SIEVE)
            checks.append({"segment": i, "start": s, "end": e, "bit_exact": got == want,
                           "oracle_s": time.perf_counter() - t1, "gpu_wall_s": t1 - t0})
    # the run keeps two batches in flight, so its value is wall-clock
    # throughput through gbc_verify_range, against the plain form's e2e
    out = {"metric": METRIC + " (full 5e13 slice)", "value": evens / res.wall_seconds / 1e9, "unit": "G evens/s",
           "segments": len(segs), "batches": res.batches, "wall_s": res.wall_seconds,
           "mtab_build_ms": st.mtab_build_ms, "plain": plain,
           "batched_over_plain": (evens / res.wall_seconds / 1e9) / plain["e2e"]["value"],
           "oracle_segments": checks, "gbstats": line,
           "config": {"workload": f"[{a}, {b}]", "segments_per_batch": args.batch,
                      "sample_every": args.sample_every}}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=12)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=0, help="segments per batch (0: the record's, else 16)")
    ap.add_argument("--sample-every", type=int, default=256)
    ap.add_argument("--tile-log2", type=int, default=0)
    ap.add_argument("--tile-bits", type=int, default=0, help="bits per tile (a multiple of 4096); overrides the record")
    ap.add_argument("--p-mid", type=int, default=0)
    ap.add_argument("--hl-mode", type=int, default=0)
    ap.add_argument("--mtab-gb", type=int, default=0)
    ap.add_argument("--launch-mode", type=int, default=0)
    ap.add_argument("--plan-funnels", type=int, default=0)
    ap.add_argument("--ref-evens", type=int, default=1_000_000)
    ap.add_argument("--cpu-evens", type=int, default=4_000_000)
    ap.add_argument("--exact-steps", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--plain-segments", type=int, default=48)
    ap.add_argument("--windows", type=int, default=256)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-sweep", default="500,2000",
                    help="more request rates (per s) for the serving loop under load, comma-separated ('': none)")
    ap.add_argument("--sweep-seconds", type=float, default=10.0)
    ap.add_argument("--slice", action="store_true")
    ap.add_argument("--sparse-segments", type=int, default=2, help="segments of the sparse leg (0: none)")
    ap.add_argument("--sparse-dlt-log2", type=int, default=26)
    ap.add_argument("--sparse-only", action="store_true", help="run the sparse leg alone and print its line")
    ap.add_argument("--tuning", default="", help="autotuner record (default: the committed one); 'none': defaults")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.slice:
        return slice_mode(args)
    if args.sparse_only:
        import gbc
        print(json.dumps(sparse_leg(gbc, args.sparse_segments, args.sparse_dlt_log2)))
        return 0
    rep = Replicas()
    try:
        return run_gb300(args, rep)
    finally:
        rep.close()


def run_gb300(args, rep):
    import gbc

    start = workload_start()
    nb = args.warmup + 2 * args.steps + 2 + args.exact_steps
    # knobs: the autotuner's record when there is one (goldbach-l0_gb300/autotune.py),
    # then every knob given on the command line (0: not given)
    knobs = {"max_batch": 16, "tile_log2": 0, "p_mid": 0, "plan_funnels": 0, "mtab_max_gb": 0}
    tuned = None
    if args.tuning != "none":
        import autotune
        tuned = autotune.load(args.tuning or autotune.DEFAULT_RECORD)
        if tuned:
            knobs.update(tuned)
    for name, v in (("max_batch", args.batch), ("tile_log2", args.tile_log2), ("p_mid", args.p_mid),
                    ("plan_funnels", args.plan_funnels), ("mtab_max_gb", args.mtab_gb), ("tile_bits", args.tile_bits)):
        if v:
            knobs[name] = v
    args.batch = knobs["max_batch"]
    # rank r: its own consecutive segments, after those of the ranks below
    allb = batches(start, rep.rank * nb * args.batch, nb, args.batch)
    limit = allb[-1][-1][2]
    evens_per_step = sum((e - s) // 2 + 1 for _, s, e in allb[0])
    with gbc.Context(limit=limit, segment_even=SEG, hl_mode=args.hl_mode, launch_mode=args.launch_mode,
                     device=rep.local, **knobs) as ctx:
        device_run(ctx, allb[:args.warmup], limit, args.sample_every, gbc)   # warm-up (builds the tables)
        launches0 = ctx.launches()
        timed = allb[args.warmup:args.warmup + args.steps]
        rep.barrier()
        with Clocks(rep.local) as clk:
            t0 = time.perf_counter()
            dev_ms, stage = device_run(ctx, timed, limit, args.sample_every, gbc)
            wall = time.perf_counter() - t0
        rep.barrier()
        dev_ms = rep.max(dev_ms)
        wall = rep.max(wall)
        launches = ctx.launches() - launches0
        value = rep.world * evens_per_step * args.steps / (dev_ms / 1e3) / 1e9
        # e2e: the caller's loop, two slots in flight, results to host memory
        off = args.warmup + args.steps
        e2eb = allb[off:off + args.steps]
        rep.barrier()
        t0 = time.perf_counter()
        for i in range(min(2, args.steps)):
            segs, flags = seg_args(e2eb[i], args.sample_every, gbc)
            ctx.enqueue_batch(i, segs, limit, flags)
        for i in range(args.steps):
            slot = i & 1
            ctx.collect(slot, len(e2eb[i]))
            if i + 2 < args.steps:
                segs, flags = seg_args(e2eb[i + 2], args.sample_every, gbc)
                ctx.enqueue_batch(slot, segs, limit, flags)
        e2e_wall = rep.max(time.perf_counter() - t0)
        e2e = rep.world * evens_per_step * args.steps / e2e_wall / 1e9
        d2h = args.batch * ctypes.sizeof(gbc.SegmentResult)
        # p(n) of every even on every segment
        exb = allb[off + args.steps + 2:off + args.steps + 2 + args.exact_steps] if rep.world == 1 else []
        ex_ms, ex_stage = device_run(ctx, exb, limit, 1, gbc)
        exact_all = evens_per_step * len(exb) / (ex_ms / 1e3) / 1e9 if exb else None
        cfg = ctx.cfg
        cst = ctx.stats()
    hbm, kind = peaks()
    # The kernels of each stage and their algorithmic bytes per launch (one
    # launch per batch: the kernels are persistent over the batch's
    # segments). A segment's class map is one bit per q coprime to 30:
    # SEG / 30 bytes. The hit-list stage reads its primes once and the table
    # bytes of their multiplier ranges and writes one 4-byte offset per
    # semiprime mark (the marks counted by the density of q = p m, p >= p_hl,
    # m prime) into region bins, then reads them back and writes them into
    # tile bins; the tile stage reads the tile bins once and writes the maps
    # once.
    import math
    seg_map = SEG / 30
    W = args.batch * SEG
    q_top = float(limit)
    p_max = math.sqrt(q_top)
    p_hl = float(cst.p_hl) if cst.p_hl else p_max
    L, u0, u1 = math.log(q_top), math.log(p_hl), math.log(p_max)
    marks = W * math.log(u1 * (L - u0) / (u0 * (L - u1))) / L if u1 > u0 else 0.0
    n_hl = NPRIMES_4E18 - p_hl / (math.log(p_hl) - 1.08366) if u1 > u0 else 0.0
    table_bytes = W / 30 * math.log(u1 / u0) if u1 > u0 else 0.0
    maps = args.batch * seg_map
    per_stage = {
        "tile": (["k_tile"], maps + 4 * marks),                                  # tile bins read, maps written
        "large": (["k_hitlist", "k_binsort"], 4 * n_hl + table_bytes + 12 * marks),
        "check": (["k_verify", "k_tail"], maps),                                 # the maps, read once
        "count": (["k_count"], maps),                                            # the maps, read once
    }
    # Shared-memory atomics per launch (algorithmic): the tile sieve clears
    # every multiple of its shared-atomic primes 71 <= p < p_mid in each of
    # the 8 class arrays (W / 30 bits each) and every hit-list mark; the
    # harvest counts each mark into its bin and the sort counts and ranks it;
    # the count kernel adds each prime's gap to the histogram.
    import numpy as np
    sieve_to = int(cfg.p_mid)
    flags_ = np.ones(sieve_to, dtype=bool)
    flags_[:2] = False
    for q_ in range(2, int(sieve_to ** 0.5) + 1):
        if flags_[q_]:
            flags_[q_ * q_::q_] = False
    inv_sum = float((1.0 / np.nonzero(flags_[71:])[0].__add__(71)).sum())
    smem_atomics = {"tile": 8 * W / 30 * inv_sum + marks, "large": 3 * marks, "check": 0.0, "count": W / L}
    counters = ncu_counters()
    # the shared-memory atomic roof: the device's conflict-free atomicAnd
    # throughput, measured after the timed region
    try:
        smem_peak, smem_peak_clk = gbc.smem_atomic_peak()
    except Exception:
        smem_peak, smem_peak_clk = None, None
    sm_mhz = clk.summary().get("sm_mhz") or 2070.0
    issue_peak = cst.sm_count * 4 * sm_mhz * 1e6                    # warp instructions per second
    stage_bw = {}
    for s_, (kerns, b) in per_stage.items():
        ms = stage[s_] / args.steps
        row = {"kernel": "+".join(kerns), "ms_per_launch": ms, "alg_bytes_per_launch": b,
               "achieved_gbs": b / (ms / 1e3) / 1e9 if ms > 0 else None,
               "frac_hbm": b / (ms / 1e3) / 1e9 / hbm if ms > 0 else None,
               "smem_atomics_per_launch": smem_atomics[s_],
               "smem_atomic_rate_g_per_s": smem_atomics[s_] / (ms / 1e3) / 1e9 if ms > 0 else None,
               "smem_atomics_per_clock_per_sm": smem_atomics[s_] / (ms / 1e3) / (cst.sm_count * sm_mhz * 1e6)
               if ms > 0 else None,
               "frac_smem_atomic": smem_atomics[s_] / (ms / 1e3) / smem_peak if ms > 0 and smem_peak else None}
        have = [counters[k] for k in kerns if k in counters]
        if have:
            row["ncu_dram_bytes_per_launch"] = sum(c[0] for c in have)
            if all(c[1] is not None for c in have):
                row["ncu_warp_inst_per_launch"] = sum(c[1] for c in have)
                row["issue_frac"] = row["ncu_warp_inst_per_launch"] / (ms / 1e3) / issue_peak if ms > 0 else None
        stage_bw[s_] = row
    dom = max(stage, key=stage.get)                     # the stage with the most device time per step
    kernel = stage_bw[dom]["kernel"]
    achieved = stage_bw[dom]["achieved_gbs"]
    traffic = stage_bw[dom].get("ncu_dram_bytes_per_launch")
    out = {
        "metric": METRIC, "value": value, "unit": "G evens/s", "n_gpus": rep.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"production segments of {SEG} integers from {start} (4e18 + k*467.5e6, k seed 1), "
                               f"{args.batch} segments per step",
                   "segments_per_step": args.batch, "evens_per_step": evens_per_step,
                   "parallelism": f"{rep.world} independent replicas (each rank its own segments, "
                                  f"a barrier and a max over ranks of the time; no collective)"
                   if rep.world > 1 else "one GPU",
                   "stats": f"every {args.sample_every}th segment p(n) of every even, the others funnel verify "
                            f"+ exact p(n) >= plan bound; primes, twins, gap walk, map hash on every segment",
                   "l2": f"inputs larger than L2: {args.batch * SEG / 30 / 1e6:.0f} MB of class maps + 393 MB "
                         f"of sieving primes per step",
                   "tile_log2": cfg.tile_log2, "tile_bits": cfg.tile_bits, "p_mid": cfg.p_mid, "hl_mode": cfg.hl_mode,
                   "mtab_max_gb": cfg.mtab_max_gb, "plan_funnels": cfg.plan_funnels,
                   "verify_funnels": cfg.verify_funnels,
                   "launch": "graph replay" if cfg.launch_mode != 2 else "direct launches",
                   "tuning": ("autotuner record " + os.path.relpath(args.tuning or autotune.DEFAULT_RECORD, ROOT))
                   if tuned else "defaults"},
        "stage_ms_per_step": {k: v / args.steps for k, v in stage.items()},
        "wall_ms_per_step": wall * 1e3 / args.steps,
        "exact_all": {"value": exact_all, "unit": "G evens/s",
                      "stage_ms_per_step": {k: v / len(exb) for k, v in ex_stage.items()} if exb else None},
        "e2e": {"value": e2e, "unit": "G evens/s", "h2d_bytes_per_step": 16 * args.batch,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": kernel, "stage": dom, "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic, "peak_kind": kind,
                     "alg_bytes_per_launch": stage_bw[dom]["alg_bytes_per_launch"],
                     "ms_per_launch": stage_bw[dom]["ms_per_launch"],
                     "issue_peak_warp_inst_per_s": issue_peak,
                     "smem_atomic_peak": {"per_s": smem_peak, "per_clock_per_sm": smem_peak_clk,
                                          "pattern": "conflict-free 32-bit atomicAnd, 1024 threads per SM "
                                                     "(gbc_smem_atomic_peak)"},
                     "stages": stage_bw},
        "clocks": clk.summary(),
    }
    if rep.world > 1:
        # N independent replicas: the headline and e2e legs only, rank 0 reports
        if rep.rank == 0:
            print(json.dumps(out))
        return 0
    if args.plain_segments:
        # the plain form as the reference runs it (hit lists once per batch of
        # segments), and one segment per batch with every stage per segment
        out["plain"] = plain_form_leg(gbc, start, nb * args.batch, knobs, args.batch)
        out["plain_one_segment_batches"] = plain_leg(gbc, start, args.plain_segments, (nb + 4) * args.batch, knobs)
        out["batched_over_plain"] = {"device": value / out["plain"]["value"],
                                     "e2e": e2e / out["plain"]["e2e"]["value"]}
    if args.windows:
        out["windows"] = windows_leg(gbc, args.windows, knobs=knobs)
        out["windows_verify"] = windows_leg(gbc, args.windows, knobs=knobs, sample_every=gbc.SAMPLE_NONE)
    if args.serve_seconds > 0:
        out["serving"] = serving_leg(gbc, args.serve_seconds, args.serve_rate, knobs=knobs)
        # the same loop under load: continuous batching as the request rate grows
        sweep = [float(x) for x in args.serve_sweep.split(",") if x.strip()]
        if sweep:
            out["serving_sweep"] = [
                {k: v for k, v in serving_leg(gbc, args.sweep_seconds, r, check=16, knobs=knobs).items() if k != "config"}
                for r in sweep]
    if args.sparse_segments:
        out["sparse"] = sparse_leg(gbc, args.sparse_segments, args.sparse_dlt_log2)
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args.cpu_evens, start)
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
