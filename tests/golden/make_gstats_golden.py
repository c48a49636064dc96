#!/usr/bin/env python3
"""Regenerates tests/golden/gstats/ from the reference's own campaign
statistics code.

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
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "gstats")
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


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_gstats")
    if not os.path.exists(exe):
        sys.exit("build the reference harness first: make -C oracle ref REF=<goldbach-l0 tree>")
    os.makedirs(OUT, exist_ok=True)
    with tempfile.TemporaryDirectory() as d:
        args = [exe, d, VERSION, str(SAMPLE_EVERY), str(SEG_EVEN)]
        for g, a, b in RUNS:
            args += [str(g), str(a), str(b)]
        subprocess.run(args, check=True)
        for i in range(1, len(RUNS) + 1):
            for ext in ("state", "gaps"):
                src = os.path.join(d, f"after{i}.{ext}")
                if os.path.exists(src):
                    shutil.copy(src, os.path.join(OUT, f"after{i}.{ext}"))
        shutil.copy(os.path.join(d, "goldbach_stats.log"), os.path.join(OUT, "goldbach_stats.log"))


if __name__ == "__main__":
    main()
