"""Ridge store, records file and the CPU re-proof (the reference's
RidgeTracker store, include/ridge.hpp, and records file + hook,
include/gstats.hpp:836-868). Host logic only, against the oracle's
p(n)."""
import os
import time

import gbc
import oracle


def rows(path):
    out = []
    for ln in path.read_text().splitlines():
        if ln.startswith("#") or not ln:
            continue
        r, n, p, q, s, t = (int(x) for x in ln.split(","))
        out.append((r, n, p, q, s, t))
    return out


def ridge_cases(a=10**15, count=200_000, floor=700):
    """(n, p(n)) of the evens from a with p(n) >= floor, by the oracle."""
    pn = oracle.pn_range(a, count)
    return [(a + 2 * i, pn[i]) for i in range(count) if pn[i] >= floor]


def test_pn_exact_matches_oracle():
    evens = list(range(6, 3000, 2)) + [4 * 10**18 + 2 * k for k in range(50)] + [10**15 + 2 * k for k in range(50)]
    for n in evens:
        assert gbc.pn_exact(n) == oracle.min_goldbach_prime(n), n


def test_ridge_store_keeps_proved_rows_in_order(tmp_path):
    st = tmp_path / "ridges.csv"
    good = ridge_cases()
    assert len(good) > 40
    n0, p0 = good[0]
    bad = [
        (n0 + 1, p0),                                          # odd "even"
        (n0, p0 + 2 if not oracle.is_prime(p0 + 2) else p0 + 4),  # p composite or not minimal
        (good[1][0], good[1][1] - 2),                           # below p(n): n - p composite or p composite
    ]
    # a claimed witness above p(n): p and n - p prime, but p(n) is smaller
    for n, p in good[2:40]:
        for pp in range(p + 2, p + 400, 2):
            if oracle.is_prime(pp) and oracle.is_prime(n - pp):
                bad.append((n, pp))
                break
    entries = [(n, p, 10**15) for n, p in good] + [(n, p, 10**15) for n, p in bad]
    kept = gbc.ridges_merge(st, entries, floor=700)
    want = sorted(good, key=lambda e: (-e[1], -e[0]))[:30]
    got = rows(st)
    assert kept == 30 == len(got)
    assert [(r[1], r[2]) for r in got] == want
    assert [r[0] for r in got] == list(range(1, 31))
    assert all(r[3] == r[1] - r[2] and r[4] == 10**15 and r[5] > 0 for r in got)


def test_ridge_store_reload_revalidates_and_keeps_found_time(tmp_path):
    st = tmp_path / "ridges.csv"
    good = ridge_cases(count=100_000)[:10]
    gbc.ridges_merge(st, [(n, p, 7) for n, p in good], floor=700)
    first = rows(st)
    time.sleep(1.1)
    # the same rows again: nothing changes, the found times stay
    gbc.ridges_merge(st, [(n, p, 7) for n, p in good], floor=700)
    assert rows(st) == first
    # a hand-edited row (p not the smallest witness) is dropped on the next load
    lines = st.read_text().splitlines()
    r, n, p, q, s, t = (int(x) for x in lines[2].split(","))
    lines[2] = f"{r},{n},{p + 2},{n - p - 2},{s},{t}"
    st.write_text("\n".join(lines) + "\n")
    extra = ridge_cases(a=10**15 + 200_000, count=100_000)[0]
    gbc.ridges_merge(st, [(extra[0], extra[1], 9)], floor=700)
    got = [(x[1], x[2]) for x in rows(st)]
    assert (n, p + 2) not in got and (n, p) not in got
    assert (extra[0], extra[1]) in got and len(got) == 10


def test_ridge_floor(tmp_path):
    st = tmp_path / "ridges.csv"
    good = ridge_cases(count=50_000, floor=500)
    kept = gbc.ridges_merge(st, [(n, p, 0) for n, p in good], floor=800)
    assert kept == min(30, sum(1 for _, p in good if p >= 800))
    assert all(r[2] >= 800 for r in rows(st))


def wait_for(path, timeout=10.0):
    t0 = time.time()
    while time.time() - t0 < timeout:
        if path.exists() and path.read_text().strip():
            return path.read_text()
        time.sleep(0.05)
    return path.read_text() if path.exists() else ""


def test_record_events_lines_check_and_hook(tmp_path):
    rec, hook_out = tmp_path / "records.txt", tmp_path / "hook.txt"
    hook = f"sh -c 'echo \"$@\" >> {hook_out}' hook"
    n = 10**15 + 123456
    p = oracle.min_goldbach_prime(n)
    gbc.record_event(rec, n, p, hook=hook)
    line = rec.read_text().splitlines()[-1]
    assert f" p(n)={p} n={n} q={n - p} cpu_check=OK  p(n) beyond the candidate list" in line
    assert wait_for(hook_out).split() == ["BEYOND", str(p), str(n), str(n - p), "OK"]
    # a claimed p(n) above 9781 that is not p(n): a RECORD line that says MISMATCH
    gbc.record_event(rec, n, 9787)
    line = rec.read_text().splitlines()[-1]
    assert "p(n)=9787" in line and "cpu_check=MISMATCH" in line and "NEW RECORD" in line


def test_sp_events_once_per_campaign(tmp_path):
    rec = tmp_path / "records.txt"
    n = 4 * 10**18 + 2
    gbc.record_event(rec, n, 8423, first=True)      # an unknown-S(p) prime: SP
    gbc.record_event(rec, n + 2, 8423, first=True)  # its S(p) is in the records file now
    gbc.record_event(rec, n, 8431, first=True)      # S(8431) is known: no event
    lines = rec.read_text().splitlines()
    assert len(lines) == 1
    assert "p(n)=8423" in lines[0] and "S(p) candidate" in lines[0] and f"n={n}" in lines[0]
    assert "cpu_check=MISMATCH" in lines[0]  # 8423 is not p(n) of this n
    assert not os.path.exists(str(rec) + ".tmp")
