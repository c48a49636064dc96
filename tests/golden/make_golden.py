#!/usr/bin/env python3
"""Regenerates the golden fixtures in this directory from the reference.

Runs only where the goldbach-l0 source tree is present (its path is the
first argument, or GB_REFERENCE) and after `make -C oracle ref REF=...` has
compiled the reference's own CPU path into oracle/_ref/. Everything it writes
is plain data; the tests read these files and never the reference itself.

  stats_ref_windows.txt  "START LIMIT<TAB>line": output of the reference's
                         tests/stats_ref.cpp on each window (8 threads).
  pn_<tag>.txt           "n p(n)" per even, from the reference's
                         gb::cpu_min_goldbach_prime (src/primes.cpp:482-493)
                         via oracle/_ref/pn_dump.
  pn_digests.txt         "START COUNT sha256": sha256 of the little-endian
                         u16 p(n) sequence of longer windows, same source.
  known_sp.txt           "p S rec": the published S(p) table embedded in the
                         reference's tests/stats_ref.cpp:35-42.
  known_windows.txt      "name S N primes pmax n_pmax": the independent
                         verifier's published windows listed in the
                         reference's tests/known_windows.py:45-53 ("-" where
                         a value is not published).
  psp2_below_2_32.txt    the base-2 Fermat pseudoprimes below 2^32, the
                         reference's tests/data/psp2_below_2_32.txt.
"""
import hashlib
import os
import re
import struct
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFBIN = os.path.join(REPO, "oracle", "_ref")

STATS_WINDOWS = [
    (1000000, 3000000),
    (1000000000000, 1000002000000),
    (4000000000000000000, 4000000000001000000),
    (4400000000000000000, 4400000000001000000),
    (4999999999999000000, 5000000000000000000),
    (9223372036853775808, 9223372036855775808),        # across 2^63
    (18446742974196923840, 18446742974197923840),      # top: 2^64 - 2^40
    (1425172824437600000, 1425172824437800000),        # gap 1476
    (804212830686600000, 804212830686800000),          # gap 1442
    (1425172824436700150, 1425172824438700150),
]

PN_WINDOWS = [                       # tag, first even, evens
    ("low", 4, 6000),
    ("1e12", 1000000000000, 3000),
    ("4e18", 4000000000000000000, 3000),
    ("top", 18446742974197917840, 3000),
]

PN_DIGESTS = [
    (4, 200000),
    (1000000000000, 200000),
    (4000000000000000000, 200000),
    (3325581707333960528 - 200000, 100001),   # ends at S(9781)
]


def run(args):
    return subprocess.run(args, check=True, capture_output=True, text=True).stdout


def pn_list(start, count):
    out = run([os.path.join(REFBIN, "pn_dump"), str(start), str(count), "8"])
    return [tuple(int(x) for x in ln.split()) for ln in out.splitlines()]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GB_REFERENCE", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py <goldbach-l0 tree> (or GB_REFERENCE=<tree>)")
    with open(os.path.join(HERE, "stats_ref_windows.txt"), "w") as f:
        for a, b in STATS_WINDOWS:
            line = run([os.path.join(REFBIN, "stats_ref"), str(a), str(b), "8"]).strip()
            f.write(f"{a} {b}\t{line}\n")
    for tag, start, count in PN_WINDOWS:
        with open(os.path.join(HERE, f"pn_{tag}.txt"), "w") as f:
            for n, p in pn_list(start, count):
                f.write(f"{n} {p}\n")
    with open(os.path.join(HERE, "pn_digests.txt"), "w") as f:
        for start, count in PN_DIGESTS:
            ps = [p for _, p in pn_list(start, count)]
            dig = hashlib.sha256(struct.pack(f"<{len(ps)}H", *ps)).hexdigest()
            f.write(f"{start} {count} {dig}\n")
    # the S(p) table embedded in stats_ref.cpp
    src = open(os.path.join(ref, "tests", "stats_ref.cpp")).read()
    with open(os.path.join(HERE, "known_sp.txt"), "w") as f:
        for p, s, rec in re.findall(r"\{(\d+),\s*(\d+)(?:ull)?,\s*(true|false)\}", src):
            f.write(f"{p} {s} {1 if rec == 'true' else 0}\n")
    # the published windows of tests/known_windows.py
    kw = open(os.path.join(ref, "tests", "known_windows.py")).read()
    body = kw[kw.index("WINDOWS = ["):]
    body = body[len("WINDOWS = "):body.index("]\n") + 1]
    # plain tuples of integer expressions (E18, 10**k) and strings
    rows = eval(body, {"__builtins__": {}, "E18": 4 * 10**18})
    with open(os.path.join(HERE, "known_windows.txt"), "w") as f:
        for name, s, n, primes, pmax, npmax, _src in rows:
            f.write(f"{name} {s} {n} {primes} {pmax if pmax else '-'} {npmax if npmax else '-'}\n")
    with open(os.path.join(ref, "tests", "data", "psp2_below_2_32.txt")) as src_f, \
            open(os.path.join(HERE, "psp2_below_2_32.txt"), "w") as f:
        for ln in src_f:
            ln = ln.strip()
            if ln and ln[0].isdigit():
                f.write(ln.split()[0] + "\n")


if __name__ == "__main__":
    main()
