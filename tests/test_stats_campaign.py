"""The campaign statistics files against the reference's own (CPU).

tests/golden/gstats/ holds what the reference's GoldbachStats (include/
gstats.hpp, compiled into oracle/_ref by tests/golden/make_gstats_golden.py)
wrote for five runs around 2^63 in production sampling (every second segment
sampled): a run merged, an adjacent run merged into one range, a repeated run
refused (GBPSAMP row), a run without gap statistics, and that run again with
gaps (a backfill: GBPSAMP + GBGAPS rows). tests/golden/gstats_gaps/ holds
three statistics-only runs (every segment sampled) around the record prime
gaps 1476 and 1442, committed out of order.
Here the same runs' per-segment results (restated from the oracle,
tests/stats_results.py) go through gbc_stats_commit; the state file, the gap
state and the log must equal the reference's byte for byte after every run.
The other tests check the refusal rules and the merge property on this
repository's implementation alone.
"""
import ctypes as C
import os

import pytest

import gbc
from conftest import golden_path
from stats_results import segment_results

T = 2**63
SEG_EVEN = 600_000
SAMPLE_EVERY = 2
RUNS = [(1, T - 10**6, T - 2), (1, T, T + 10**6), (1, T - 10**6, T - 2),
        (0, T + 10**6 + 2, T + 1_400_000), (1, T + 10**6 + 2, T + 1_400_000)]
MERGED = [True, True, False, True, False]
# (fixture directory, segments sampled every, segment integers, runs (gaps on, start, limit), merged)
SCENARIOS = {
    "gstats": (SAMPLE_EVERY, SEG_EVEN, RUNS, MERGED),
    "gstats_gaps": (1, 100_000, [(1, 1425172824437600000, 1425172824437800000),
                                 (1, 804212830686600000, 804212830686800000),
                                 (1, 804212830686800002, 804212830687000000)], [True, True, True]),
}


@pytest.fixture(scope="module")
def results():
    return {(a, b): segment_results(a, b, SEG_EVEN, SAMPLE_EVERY) for _, a, b in RUNS}


def commit(lib, state, log, gaps, a, b, segs, version="gb300-1.0"):
    arr = (gbc.SegmentResult * len(segs))(*segs)
    line = C.create_string_buffer(1 << 16)
    err = C.create_string_buffer(512)
    merged = C.c_int(-1)
    rc = lib.gbc_stats_commit(str(state).encode(), str(log).encode(), version.encode(), gaps, a, b, arr, len(segs),
                              line, len(line), C.byref(merged), err, len(err))
    return rc, line.value.decode(), merged.value, err.value.decode()


def read(p):
    with open(p, "rb") as f:
        return f.read()


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_statistics_files_equal_the_references(tmp_path, name):
    every, seg, runs, merged_want = SCENARIOS[name]
    lib = gbc.load()
    state, log = tmp_path / "goldbach_stats.state", tmp_path / "goldbach_stats.log"
    for i, (g, a, b) in enumerate(runs, 1):
        rc, line, merged, err = commit(lib, state, log, g, a, b, segment_results(a, b, seg, every))
        assert rc == 0, err
        assert merged == merged_want[i - 1]
        assert read(state) == read(golden_path(f"{name}/after{i}.state")), f"state after run {i}"
        gp = golden_path(f"{name}/after{i}.gaps")
        if os.path.exists(gp):
            assert read(str(state) + ".gaps") == read(gp), f"gap state after run {i}"
    assert read(log) == read(golden_path(f"{name}/goldbach_stats.log"))


def test_adjacent_runs_merge_to_one_run(tmp_path):
    """Every segment sampled: two adjacent runs merged one after the other
    leave the same state, gap state and first occurrences as one run over
    both."""
    lib = gbc.load()
    a, m, b = T - 400_000, T - 2, T + 400_000
    one, two = tmp_path / "one", tmp_path / "two"
    one.mkdir()
    two.mkdir()
    rc, _, merged, err = commit(lib, one / "s", one / "l", 1, a, b, segment_results(a, b, SEG_EVEN, 1))
    assert rc == 0 and merged == 1, err
    for x, y in ((a, m), (m + 2, b)):
        rc, _, merged, err = commit(lib, two / "s", two / "l", 1, x, y, segment_results(x, y, SEG_EVEN, 1))
        assert rc == 0 and merged == 1, err
    assert read(one / "s") == read(two / "s")
    assert read(one / "s.gaps") == read(two / "s.gaps")


def test_overlap_and_damage_are_refused(tmp_path, results):
    lib = gbc.load()
    state, log = tmp_path / "s", tmp_path / "l"
    g, a, b = RUNS[0]
    assert commit(lib, state, log, g, a, b, results[(a, b)])[0] == 0
    before = read(state)
    # overlapping a covered range: nothing merged, the state unchanged
    rc, _, merged, _ = commit(lib, state, log, g, a, b, results[(a, b)])
    assert rc == 0 and merged == 0 and read(state) == before
    # a damaged record, a cut-off file, a missing record, another tail bound
    x, y = RUNS[1][1], RUNS[1][2]
    for bad in (before.replace(b"\nevens ", b"\nevens x"), before[:-10], before.replace(b"tailagg", b"#tailagg"),
                before.replace(b"tail_t 3000", b"tail_t 2000")):
        state.write_bytes(bad)
        rc, _, _, err = commit(lib, state, log, 1, x, y, results[(x, y)])
        assert rc == -5 and ("refusing" in err or "tail_t" in err), err
        assert read(state) == bad
    # a damaged gap state is refused too
    state.write_bytes(before)
    gp = tmp_path / "s.gaps"
    gp.write_bytes(read(gp).replace(b"\nend\n", b"\n"))
    rc, _, _, err = commit(lib, state, log, 1, x, y, results[(x, y)])
    assert rc == -5 and "gap state" in err
    assert read(state) == before


def test_results_that_do_not_cover_the_run_are_rejected(tmp_path, results):
    lib = gbc.load()
    g, a, b = RUNS[1]
    segs = results[(a, b)]
    rc, _, _, err = commit(lib, tmp_path / "s", tmp_path / "l", g, a, b + 2, segs)
    assert rc == -1 and "cover" in err
    rc, _, _, err = commit(lib, tmp_path / "s", tmp_path / "l", g, a, b, segs[1:])
    assert rc == -1
    assert not (tmp_path / "s").exists()
