#!/usr/bin/env python3
"""Regenerates tests/golden/gstats/ and tests/golden/gstats_gaps/ from the
reference's own campaign statistics code.

Runs oracle/_ref/ref_gstats (oracle/ref_gstats.cpp compiled against the
reference's include/gstats.hpp by `make -C oracle ref REF=<goldbach-l0 tree>`)
on the scenario below and keeps what the reference writes:

  after<i>.state / after<i>.gaps   the state file and the gap state after run i
  goldbach_stats.log               every line the five runs appended

The scenario (segments of SEG_EVEN integers, every SAMPLE_EVERY-th sampled):
  1  [2^63 - 1e6, 2^63 - 2]          gaps on: merged
  2  [2^63, 2^63 + 1e6]              gaps on: adjacent, merged (one range)
  3  run 1 again                     overlaps: refused, a GBPSAMP row
  4  [2^63 + 1e6 + 2, 2^63 + 1.4e6]  gaps off: merged without gap statistics
  5  run 4 again, gaps on            overlaps: a GBPSAMP row, its gaps merged
                                     into the gap state (a backfill), a GBGAPS row

gstats_gaps/: every segment sampled (a statistics-only run), segments of
SEG_EVEN_GAPS integers, around the record prime gaps 1476 and 1442 (every gap
>= 700 is listed in the lines and the gap state), committed out of order:
  1  [1425172824437600000, +2e5]     the gap of 1476
  2  [804212830686600000, +2e5]      the gap of 1442, below run 1
  3  [804212830686800002, ..800000]  adjacent to run 2
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
VERSION = "gb300-1.0"
SAMPLE_EVERY = 2
SEG_EVEN = 600_000
T = 2**63
RUNS = [
    (1, T - 10**6, T - 2),
    (1, T, T + 10**6),
    (1, T - 10**6, T - 2),
    (0, T + 10**6 + 2, T + 1_400_000),
    (1, T + 10**6 + 2, T + 1_400_000),
]
SEG_EVEN_GAPS = 100_000
RUNS_GAPS = [
    (1, 1425172824437600000, 1425172824437800000),
    (1, 804212830686600000, 804212830686800000),
    (1, 804212830686800002, 804212830687000000),
]
SCENARIOS = [("gstats", SAMPLE_EVERY, SEG_EVEN, RUNS), ("gstats_gaps", 1, SEG_EVEN_GAPS, RUNS_GAPS)]


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_gstats")
    if not os.path.exists(exe):
        sys.exit("build the reference harness first: make -C oracle ref REF=<goldbach-l0 tree>")
    for name, every, seg, runs in SCENARIOS:
        out = os.path.join(HERE, name)
        os.makedirs(out, exist_ok=True)
        with tempfile.TemporaryDirectory() as d:
            args = [exe, d, VERSION, str(every), str(seg)]
            for g, a, b in runs:
                args += [str(g), str(a), str(b)]
            subprocess.run(args, check=True)
            for i in range(1, len(runs) + 1):
                for ext in ("state", "gaps"):
                    src = os.path.join(d, f"after{i}.{ext}")
                    if os.path.exists(src):
                        shutil.copy(src, os.path.join(out, f"after{i}.{ext}"))
            shutil.copy(os.path.join(d, "goldbach_stats.log"), os.path.join(out, "goldbach_stats.log"))


if __name__ == "__main__":
    main()
