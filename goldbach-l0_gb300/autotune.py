"""Autotuner of the batched form (the knobs the reference fixes by hand in
include/config.hpp: SMEM tile size, the tile / large-prime split, the
hit-list split through the prime-multiplier table's budget, segments per
batch, the verify plan's funnel count and how many of them every word takes
before the unresolved words are gathered). A table budget below what the
hit lists need from p_mid on leaves the primes between p_mid and the hit
lists to the packed large-prime tier, so the (p_mid, budget) knob also
decides how much work that tier gets.

Coordinate descent on calibration batches of the workload: from the
defaults, each knob in turn takes the value with the highest throughput
while the others stay fixed, until a round changes nothing (at most three);
p_mid and the table budget move together, since the budget decides whether
the hit lists can start at p_mid. Every trial verifies the same
consecutive production segments (192 of them, whole batches for every
batch size tried), timed on the device with the pipeline's own CUDA events, one
slot, after a warm-up batch that builds the tables. The record holds every
trial and the choice; callers (bench.py, the serving setup) load it with
`load()`.

    python goldbach-l0_gb300/autotune.py --start 4000008233142500000 \\
        --out goldbach-l0_gb300/tuning/gb300_production_4e18.json
"""
import argparse
import datetime
import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import gbc  # noqa: E402

SEG = 467_500_000
KNOBS = {
    # the tile / hit-list split and the table budget that sets where the hit
    # lists start: one joint knob (a small budget pushes p_hl above p_mid)
    ("p_mid", "mtab_max_gb"): [(p, g) for p in (1 << 20, 1638400, 1703936, 1769472, 1835008, 1 << 21, 1 << 22, 1 << 23)
                               for g in (16, 24, 48, 96, 160)],
    "tile_log2": [19, 20],
    "tile_bits": [0, 1572864, 1835008],  # 0: 2^tile_log2 bits
    "max_batch": [32, 48, 64, 96, 128],
    "plan_funnels": [6, 8, 12, 16],
    "verify_funnels": [2, 3, 4],
}
DEFAULTS = {"p_mid": 1 << 22, "mtab_max_gb": 48, "tile_log2": 20, "tile_bits": 0, "max_batch": 16,
            "plan_funnels": 8, "verify_funnels": 3}
DEFAULT_RECORD = os.path.join(HERE, "tuning", "gb300_production_4e18.json")


def measure(knobs, start, nseg=192, sample_every=256):
    """Device throughput (G evens/s) of about nseg production segments from
    start (whole batches, at least one) under the given knobs; segment i
    gets p(n) of every even when i is a multiple of sample_every, else the
    funnel verify + exact tail."""
    mb = knobs["max_batch"]
    nseg = mb * max(1, round(nseg / mb))
    segs = [(start + i * SEG, start + i * SEG + SEG - 2) for i in range(nseg + mb)]
    limit = segs[-1][1]
    flags = [0 if i % sample_every == 0 else gbc.SEG_VERIFY for i in range(len(segs))]
    with gbc.Context(limit=limit, segment_even=SEG, **knobs) as ctx:
        ctx.enqueue_batch(0, segs[:mb], limit, flags[:mb])        # warm-up: tables and the slot's graph
        ctx.collect(0, mb)
        ms = 0.0
        for b in range(mb, mb + nseg, mb):
            ctx.enqueue_batch(0, segs[b:b + mb], limit, flags[b:b + mb])
            _, t = ctx.collect(0, mb)
            ms += t.ms_total
    return nseg * (SEG // 2) / (ms / 1e3) / 1e9


def gpu_name():
    try:
        return subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader", "-i", "0"],
                              capture_output=True, text=True, timeout=20).stdout.strip()
    except Exception:
        return "unknown"


def tune(start, rounds=3, nseg=192, log=print, init=None):
    """Coordinate descent from init (default: DEFAULTS)."""
    best = dict(DEFAULTS)
    best.update(init or {})
    trials = []
    cache = {}

    def run(k):
        key = tuple(sorted(k.items()))
        if key not in cache:
            t0 = time.perf_counter()
            try:
                v = measure(k, start, nseg)
            except gbc.GbcError as e:   # e.g. the device memory of a large batch
                log(f"  {k} failed: {e}")
                v = 0.0
            cache[key] = v
            trials.append({"knobs": dict(k), "g_evens_s": v, "seconds": time.perf_counter() - t0})
            log(f"  {k} -> {v:.2f} G evens/s")
        return cache[key]

    base = run(best)
    def get(k, name):
        return tuple(k[n] for n in name) if isinstance(name, tuple) else k[name]

    def put(k, name, v):
        if isinstance(name, tuple):
            k.update(zip(name, v))
        else:
            k[name] = v

    for r in range(rounds):
        changed = False
        for name, values in KNOBS.items():
            scores = {}
            for v in values:
                k = dict(best)
                put(k, name, v)
                scores[v] = run(k)
            pick = max(scores, key=scores.get)
            if pick != get(best, name):
                put(best, name, pick)
                changed = True
        if not changed:
            break
    return {"gpu": gpu_name(), "date": datetime.datetime.now(datetime.timezone.utc).isoformat(timespec="seconds"),
            "workload": {"start": start, "segment": SEG, "segments": nseg, "sample_every": 256,
                         "what": "consecutive production segments, funnel verify + exact tail, every 256th "
                                 "segment p(n) of every even"},
            "method": "coordinate descent over the knobs ((p_mid, table budget) as one), up to three rounds, "
                      "device time of the pipeline's events",
            "defaults": DEFAULTS, "start_knobs": dict(init or DEFAULTS), "default_g_evens_s": base,
            "choice": best, "choice_g_evens_s": cache[tuple(sorted(best.items()))], "trials": trials}


def load(path=DEFAULT_RECORD):
    """The recorded choice (a dict of Context keyword arguments), or None."""
    try:
        with open(path) as f:
            return dict(json.load(f)["choice"])
    except (OSError, KeyError, ValueError):
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--start", type=int, default=4000008233142500000)
    ap.add_argument("--segments", type=int, default=192)
    ap.add_argument("--rounds", type=int, default=3)
    ap.add_argument("--out", default=DEFAULT_RECORD)
    ap.add_argument("--from-record", default="", help="start the descent from this record's choice")
    a = ap.parse_args()
    rec = tune(a.start, a.rounds, a.segments, init=load(a.from_record) if a.from_record else None)
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps({"choice": rec["choice"], "g_evens_s": rec["choice_g_evens_s"],
                      "default_g_evens_s": rec["default_g_evens_s"], "trials": len(rec["trials"])}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
