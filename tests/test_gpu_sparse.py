"""Sparse class map on the GPU against the oracle (the reference's
debug_sparse validation, docs/HISTORY.md section 9.2k: the map against an
independent CPU sieve of the same progressions and Miller-Rabin checks; the
checker against a per-even CPU reference of the plan, its pending set
exactly; forced leftovers; ragged windows across segments)."""
import random

import pytest

import gbc
import oracle
import sparse_oracle as so

pytestmark = pytest.mark.gpu

M = so.M


def rows_equal(sp, n0, dl, want_rows):
    got = sp.map(n0, dl)
    for k in range(sp.K):
        w = so.to_words(want_rows[k])
        assert got[k] == w, f"class {k}: {sum(a != b for a, b in zip(got[k], w))} words differ"


def test_map_bit_exact_1e15_two_tiles():
    # 2^20 + 4321 evens per class: two tiles per row; sieving primes to 3.2e7,
    # so both the tile kernel and the large-prime kernel mark
    n0 = 10**15 - 10**15 % M
    dl = (1 << 20) + 4321
    with gbc.Sparse(limit=n0 + M * (dl + 10), dlt_log2=21) as sp:
        rows_equal(sp, n0, dl, so.class_map(n0, dl, sp.tb, sp.residues))


def test_map_bit_exact_1e12():
    n0 = 10**12 - 10**12 % M + 7 * M
    with gbc.Sparse(limit=2 * 10**12, dlt_log2=16) as sp:
        rows_equal(sp, n0, 3000, so.class_map(n0, 3000, sp.tb, sp.residues))


@pytest.fixture(scope="module")
def sp4e18():
    with gbc.Sparse(limit=4 * 10**18 + 10**12, dlt_log2=20) as sp:
        yield sp


def test_map_every_bit_by_miller_rabin_4e18(sp4e18):
    sp = sp4e18
    n0 = 4 * 10**18 - 4 * 10**18 % M + 12345 * M
    rows_equal(sp, n0, 4096, so.map_by_mr(n0, 4096, sp.tb, sp.residues))


def test_witness_follows_the_plan_4e18(sp4e18):
    sp = sp4e18
    start = 4 * 10**18 + 2 * 98765
    count = 6000
    got = sp.witness(start, count)
    plans = {}
    for j in range(count):
        n = start + 2 * j
        r = (n % M)
        if r not in plans:
            plans[r] = [p for p, _ in sp.plan(r)]
        want = so.first_witness(n, plans[r])
        assert got[j] == want, (n, got[j], want)
        assert oracle.is_prime(got[j]) and oracle.is_prime(n - got[j])


def test_verify_ragged_windows_across_segments(sp4e18):
    sp = sp4e18
    D = M * sp.dlt
    start = 4 * 10**18 + 1234566
    limit = start + 2 * D + 777776
    r = sp.verify(start, limit)
    assert r.evens == (limit - start) // 2 + 1
    assert r.segments == len(range(start - start % M, limit + 1, D))
    assert r.pending == len(sp.pending())
    assert r.map_primes > 0 and r.groups > 0 and r.ms_check > 0
    # odd bounds round inwards
    r2 = sp.verify(start + 1, start + 2 * 5000 + 1)
    assert r2.evens == 5000


def test_forced_leftovers_match_the_oracle():
    # one candidate group per even class: the GPU must leave exactly the
    # evens whose first group holds no witness, and the CPU resolves them
    start = 4 * 10**18 + 10**9
    count = 40000
    limit = start + 2 * (count - 1)
    with gbc.Sparse(limit=4 * 10**18 + 10**12, dlt_log2=16, group_cap=1) as sp:
        r = sp.verify(start, limit)
        pend = sp.pending()
        want = []
        firsts = {}
        for j in range(count):
            n = start + 2 * j
            cls = n % M
            if cls not in firsts:
                firsts[cls] = [p for p, g in sp.plan(cls) if g == 0]
            if not so.first_witness(n, firsts[cls]):
                want.append(n)
        assert pend == want
        assert r.pending == len(want) > 0 and r.evens == count
        w = sp.witness(start, count)
        assert [start + 2 * j for j in range(count) if w[j] == 0] == want


def test_rejects_low_start_and_high_limit():
    with gbc.Sparse(limit=10**12, dlt_log2=14) as sp:
        with pytest.raises(gbc.GbcError) as e:
            sp.verify(10**6, 2 * 10**6)
        assert e.value.code == -1 and "dense path" in str(e.value)
        with pytest.raises(gbc.GbcError) as e:
            sp.verify(10**12 - 1000, 10**12 + 1000)
        assert e.value.code == -1
        r = sp.verify(10**12 - 2 * 10**6, 10**12)
        assert r.evens == 10**6 + 1


def test_cli_sparse_run():
    import os
    import subprocess
    from conftest import ROOT
    exe = os.path.join(ROOT, "goldbach-l0_gb300", "bin", "goldbach_gb300")
    r = subprocess.run([exe, "--start", "4e18", "--limit", "4000000002000000001", "--sparse", "--csv"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    kv = dict(x.split("=", 1) for x in r.stdout.strip().split(","))
    assert kv["result"] == "PASS" and kv["path"] == "sparse"
    assert int(kv["evens"]) == 10**9 + 1 and int(kv["start"]) == 4 * 10**18



def test_sparse_journaled_slices(tmp_path, sp4e18):
    # ci/sparse_crosscheck.sh run: the dense runner's rows, resume and stop file
    sp = sp4e18
    j = tmp_path / "range-sparse.journal"
    a = 4 * 10**18 + 10**10
    b = a + 3 * 10**9 - 2
    assert sp.run_slices(a, b, 10**9, j) == (3, False)
    rows = j.read_text().splitlines()
    assert len(rows) == 3
    for row, lo in zip(rows, (a, a + 10**9, a + 2 * 10**9)):
        t = row.split()
        kv = dict(x.split("=", 1) for x in t[4:] if "=" in x)
        assert t[0] == "PASS" and int(t[1]) == lo and int(t[2]) == lo + 10**9 - 2
        assert kv["path"] == "sparse" and kv["result"] == "PASS" and kv["release"] == "gb300-1.0"
        assert int(kv["start"]) == lo and int(kv["limit"]) == lo + 10**9 - 2
    assert gbc.journal_resume(j, a) == b + 2
    assert sp.run_slices(a, b, 10**9, j) == (0, False)       # resumed past the chain
    stop = tmp_path / "STOP"
    stop.write_text("")
    assert sp.run_slices(a, b + 10**9, 10**9, j, stop_file=stop) == (0, True)
    assert len(j.read_text().splitlines()) == 3
