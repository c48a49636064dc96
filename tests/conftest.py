import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "goldbach-l0_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def golden_path(name):
    return os.path.join(GOLDEN, name)


def stats_windows():
    """(start, limit, stats_ref line) of tests/golden/stats_ref_windows.txt."""
    out = []
    with open(golden_path("stats_ref_windows.txt")) as f:
        for ln in f:
            head, line = ln.rstrip("\n").split("\t")
            a, b = head.split()
            out.append((int(a), int(b), line))
    return out


def pn_fixture(tag):
    ns, ps = [], []
    with open(golden_path(f"pn_{tag}.txt")) as f:
        for ln in f:
            n, p = ln.split()
            ns.append(int(n))
            ps.append(int(p))
    return ns, ps


def pn_digests():
    with open(golden_path("pn_digests.txt")) as f:
        return [(int(a), int(b), c) for a, b, c in (ln.split() for ln in f)]


def known_sp():
    with open(golden_path("known_sp.txt")) as f:
        return [(int(p), int(s), r == "1") for p, s, r in (ln.split() for ln in f)]


def known_windows():
    rows = []
    with open(golden_path("known_windows.txt")) as f:
        for ln in f:
            name, s, n, primes, pmax, npmax = ln.split()
            rows.append((name, int(s), int(n), int(primes), None if pmax == "-" else int(pmax),
                         None if npmax == "-" else int(npmax)))
    return rows
