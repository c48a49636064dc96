"""The batched forms on the GPU: many windows of different widths and
heights in shared batches (one persistent launch per stage over all their
runs and segments), the pipeline replayed as a CUDA graph against the same
kernels launched one by one, the map self-check, and the serving loop with
each result the same alone and in the mix.

Everything is compared bit-exact: with the oracle's exact sieve (the
stats_ref line of tests/stats_ref.cpp), with Miller-Rabin for every map bit,
and with runs of each window alone through the plain per-range call.
"""
import random
import threading

import pytest

import gbc
import oracle

pytestmark = pytest.mark.gpu

U30 = [1, 7, 11, 13, 17, 19, 23, 29]

# windows at very different heights; two overlap, one is tiny, one starts at 6
WINDOWS = [
    (10**12, 10**12 + 2_400_000),
    (4 * 10**18 + 123_456, 4 * 10**18 + 1_123_456),
    (9223372036853775808, 9223372036853775808 + 600_000),
    (10**15 + 2, 10**15 + 2_999_998),
    (6, 150_000),
    (10**12 + 1_000_000, 10**12 + 3_000_000),
    (10**10, 10**10 + 10),
    (gbc.MAX_LIMIT - 1_000_000, gbc.MAX_LIMIT),
]


@pytest.fixture(scope="module")
def wctx():
    with gbc.Context(limit=gbc.MAX_LIMIT, segment_even=1_000_000, max_batch=8, max_runs=8, nslots=3) as c:
        yield c


def test_windows_in_shared_batches_match_oracle(wctx):
    """Every window's statistics from shared batches equal the oracle's."""
    out, summ = wctx.verify_windows(WINDOWS)
    assert summ.segments == sum(len(gbc.segments_of(a, b, 1_000_000)) for a, b in WINDOWS)
    assert summ.batches < summ.segments  # segments of different windows shared batches
    for (a, b), (res, line) in zip(WINDOWS, out):
        assert line == oracle.stats_line(a, b, oracle.SIEVE), (a, b)


def test_windows_equal_alone(wctx):
    """The same window alone (the plain per-range call) gives the same line."""
    out, _ = wctx.verify_windows(WINDOWS[::-1])
    for (a, b), (_, line) in zip(WINDOWS[::-1], out):
        assert line == wctx.verify_range(a, b)[1], (a, b)


def test_runs_class_maps_bit_exact():
    """Three runs at three heights in one batch: every bit of every run's
    class map against Miller-Rabin."""
    segs = [(10**12, 10**12 + 299_998), (10**12 + 300_000, 10**12 + 599_998),
            (4 * 10**18, 4 * 10**18 + 299_998), (2**63 + 10**6, 2**63 + 10**6 + 299_998)]
    limits = [10**12 + 599_998, 10**12 + 599_998, 4 * 10**18 + 299_998, 2**63 + 10**6 + 299_998]
    with gbc.Context(limit=gbc.MAX_LIMIT, segment_even=300_000, max_batch=4, max_runs=4, hl_mode=1,
                     mtab_max_gb=8, p_mid=1 << 18) as c:
        c.enqueue_segments(0, segs, limits)
        res, t = c.collect(0, len(segs))
        assert t.runs == 3
        for run in range(3):
            base, nblk, wpc, w = c.map(0, run)
            bad = [base + 30 * t + U30[k] for k in range(8) for t in range(nblk)
                   if ((w[k * wpc + (t >> 5)] >> (t & 31)) & 1) != oracle.is_prime(base + 30 * t + U30[k])]
            assert not bad, (run, bad[:8])
        with pytest.raises(gbc.GbcError):
            c.map(0, 3)


def test_graph_replay_equals_direct_launches():
    """launch_mode 1 (graph per slot) and 2 (kernels one by one) agree, and
    the graph path really replays."""
    a, b = 4 * 10**18, 4 * 10**18 + 8_000_000
    lines = []
    for mode in (1, 2):
        with gbc.Context(limit=b, segment_even=1_000_000, max_batch=4, hl_mode=1, mtab_max_gb=8,
                         launch_mode=mode) as c:
            lines.append(c.verify_range(a, b)[1])
            st = c.stats()
            assert st.batches == 3
            assert st.graph_replays == (3 if mode == 1 else 0)
    assert lines[0] == lines[1] == oracle.stats_line(a, b, oracle.SIEVE)


def test_map_selfcheck_runs_and_passes():
    """Every batch rebuilt without hit lists and compared word for word."""
    a, b = 9 * 10**18, 9 * 10**18 + 6_000_000
    with gbc.Context(limit=b, segment_even=1_000_000, max_batch=2, hl_mode=1, mtab_max_gb=8,
                     selfcheck_every=1) as c:
        line = c.verify_range(a, b)[1]
        st = c.stats()
    assert st.selfchecks == st.batches == 4
    assert line == oracle.stats_line(a, b, oracle.SIEVE)


@pytest.mark.parametrize("tile_bits", [1835008, 1572864])
def test_tiles_across_hit_list_regions_selfcheck(tile_bits):
    """Tiles of any size (not a power of two) in a one-run batch of 20
    production segments at 4e18: each class array spans two hit-list regions
    of 2^28 bits, a tile straddles their border, and its bin is filled from
    both. The maps equal the rebuild without hit lists word for word
    (self-check), and the map hash of three segments equals the oracle's."""
    seg = 467_500_000
    a = 4000008233142500000
    segs = [(a + i * seg, a + (i + 1) * seg - 2) for i in range(20)]
    limit = segs[-1][1]
    with gbc.Context(limit=limit, segment_even=seg, max_batch=20, p_mid=1 << 21, mtab_max_gb=96, hl_mode=1,
                     tile_bits=tile_bits, selfcheck_every=1) as c:
        c.enqueue_batch(0, segs, limit, [0] + [gbc.SEG_VERIFY] * 19)
        res, _ = c.collect(0, 20)
        assert c.stats().selfchecks == 1 and c.stats().p_hl > 0
    nblk = (segs[-1][1] + 3 - (a - 9781) // 30 * 30) // 30 + 1
    assert nblk > 1 << 28
    for r in (res[0], res[9], res[19]):
        assert (r.map_hash, r.map_primes) == oracle.map_hash(r.hash_lo, r.hash_hi)


def test_packed_large_tier_selfcheck_production():
    """The packed large-prime tier active between p_mid = 2^21 and the hit
    lists (a 24 GB multiplier table puts p_hl near 5.6e6): two production
    segments at 4e18, the map equal to the rebuild without hit lists word for
    word, the hashes and the first segment's statistics equal the oracle's."""
    seg = 467_500_000
    a = 4000008233142500000
    segs = [(a, a + seg - 2), (a + seg, a + 2 * seg - 2)]
    limit = segs[-1][1]
    with gbc.Context(limit=limit, segment_even=seg, max_batch=2, p_mid=1 << 21, mtab_max_gb=24, hl_mode=1,
                     selfcheck_every=1) as c:
        assert c.stats().p_hl > 5_000_000
        c.enqueue_batch(0, segs, limit, [0, gbc.SEG_VERIFY])
        res, _ = c.collect(0, 2)
        assert c.stats().selfchecks == 1
    for r in res:
        assert (r.map_hash, r.map_primes) == oracle.map_hash(r.hash_lo, r.hash_hi)


def result_fields(r):
    """A segment result as comparable fields; the lists the kernels append
    to with atomics (leftovers, gap tails, ridges) in no fixed order, as
    sorted lists."""
    import ctypes as C
    out = {}
    lists = {"left_n": "nleft", "left_p": "nleft", "tail_g": "ntail", "tail_lo": "ntail", "ridge_p": "nridge",
             "ridge_n": "nridge"}
    for name, _ in gbc.SegmentResult._fields_:
        v = getattr(r, name)
        if name in lists:
            continue
        out[name] = C.string_at(C.addressof(v), C.sizeof(v)) if hasattr(v, "_length_") else v
    out["left"] = sorted(zip(r.left_n[:r.nleft], r.left_p[:r.nleft]))
    out["tail"] = sorted(zip(r.tail_lo[:r.ntail], r.tail_g[:r.ntail]))
    out["ridges"] = sorted(zip(r.ridge_n[:r.nridge], r.ridge_p[:r.nridge]))
    return out


@pytest.mark.parametrize("tile_bits", [0, 1835008])
def test_plain_form_equals_batched_form(tile_bits):
    """The plain form (launch mode 3: hit lists harvested once for the
    batch, then each segment through its own launches of the sieve, the
    packed large primes, the checkers and the counts) gives every segment
    the same results, byte for byte, as the batched form's graph replay:
    four production segments at 4e18 with the packed tier and the hit lists
    on, production sampling; the map hashes equal the oracle's."""
    seg = 467_500_000
    a = 4000008233142500000
    segs = [(a + i * seg, a + (i + 1) * seg - 2) for i in range(4)]
    limit = segs[-1][1]
    flags = [0, gbc.SEG_VERIFY, gbc.SEG_VERIFY, gbc.SEG_VERIFY]
    out = {}
    for mode in (1, 3):
        with gbc.Context(limit=limit, segment_even=seg, max_batch=4, p_mid=1 << 21, mtab_max_gb=24, hl_mode=1,
                         tile_bits=tile_bits, launch_mode=mode) as c:
            c.enqueue_batch(0, segs, limit, flags)
            res, _ = c.collect(0, 4)
            out[mode] = [result_fields(r) for r in res]
            if mode == 3:
                for r in res:
                    assert (r.map_hash, r.map_primes) == oracle.map_hash(r.hash_lo, r.hash_hi)
    for i, (x, y) in enumerate(zip(out[1], out[3])):
        assert x == y, (i, [k for k in x if x[k] != y[k]])


def test_prepare_builds_the_table_once():
    with gbc.Context(limit=5 * 10**18, segment_even=1_000_000, max_batch=4, hl_mode=1, mtab_max_gb=16) as c:
        c.prepare(10**16, 5 * 10**18)
        assert c.stats().mtab_builds == 1
        for a in (10**16, 10**17 + 8, 3 * 10**18, 5 * 10**18 - 4_000_000):
            c.verify_range(a, a + 3_000_000)
        assert c.stats().mtab_builds == 1


def serving_windows(n, seed):
    rnd = random.Random(seed)
    out = []
    for _ in range(n):
        a = int(10 ** rnd.uniform(10, 18.6)) // 2 * 2
        w = int(10 ** rnd.uniform(4, 6.5)) // 2 * 2
        out.append((a, a + w))
    return out


@pytest.mark.parametrize("sample_every", [1, 2])
def test_server_results_same_alone_and_in_the_mix(sample_every):
    """Windows submitted from several threads while others are on the GPU:
    each window's line equals its line alone (bit-exact, no tolerance), and
    several batches were in flight at once."""
    wins = serving_windows(40, 11 + sample_every)
    with gbc.Context(limit=gbc.MAX_LIMIT, segment_even=1_000_000, max_batch=8, nslots=4,
                     sample_every=sample_every) as c:
        got = {}
        with gbc.Server(c, hbm_budget=150 * 10**9) as srv:
            tickets = {}

            def submit(part):
                for w in part:
                    tickets[w] = srv.submit(*w)

            th = [threading.Thread(target=submit, args=(wins[i::4],)) for i in range(4)]
            for t in th:
                t.start()
            for t in th:
                t.join()
            for w, tk in tickets.items():
                got[w] = srv.wait(tk)
            st = srv.stats()
        assert st.completed == len(wins)
        assert st.segments >= len(wins)
        for w in wins:
            res, line, lat = got[w]
            assert lat > 0
            assert line == c.verify_range(*w)[1], w
        for w in wins[:4]:
            if sample_every == 1:
                assert got[w][1] == oracle.stats_line(w[0], w[1], oracle.SIEVE)


def test_plain_1e12_window_config_c1():
    """All evens in [1e12, 1e12 + 1e9] through the plain form (one segment
    per batch, tile + mid stages only at this height) against the oracle's
    exact sieve: the whole stats_ref line (every p(n), primes, twins, gaps)."""
    a, b = 10**12, 10**12 + 10**9
    with gbc.Context(limit=b, segment_even=100_000_000, max_batch=1, launch_mode=2) as c:
        res, line, _ = c.verify_range(a, b)
        assert c.stats().p_hl == 0  # no hit lists below 1e13
    assert res.evens == 500_000_001
    assert line == oracle.stats_line(a, b, oracle.SIEVE)


def uneven_windows(n=256, seed=7):
    """The batched uneven-window workload: widths log-uniform in [1e6, 1e10],
    starts uniform in [1e15, 5e18], both even (seed 7)."""
    import math
    rnd = random.Random(seed)
    out = []
    for _ in range(n):
        w = int(math.exp(rnd.uniform(math.log(1e6), math.log(1e10)))) // 2 * 2
        a = int(rnd.uniform(1e15, 5e18)) // 2 * 2
        out.append((a, a + w))
    return out


def test_uneven_windows_sampled_against_oracle_config_c4():
    """All 256 windows in shared batches, plus one of 1e9 across 2^63;
    against the oracle's exact sieve: 8 sampled windows (seed 8, among those
    under 2e7 wide so the oracle finishes in seconds), the narrowest window
    of at least 1e9 (several 467.5M segments in one run) and the window
    across 2^63; every one of 16 sampled windows against its run alone."""
    wins = uneven_windows()
    small = [i for i, (a, b) in enumerate(wins) if b - a < 2 * 10**7]
    pick = random.Random(8).sample(small, 8)
    wide = min((i for i, (a, b) in enumerate(wins) if b - a >= 10**9), key=lambda i: wins[i][1] - wins[i][0])
    top = 2**63 - 400_000_000
    wins.append((top, top + 10**9))
    pick += [wide, len(wins) - 1]
    limit = max(b for _, b in wins)
    with gbc.Context(limit=limit, segment_even=gbc.DEFAULT_SEGMENT, max_batch=16, max_runs=16, nslots=3) as c:
        out, summ = c.verify_windows(wins)
        assert summ.runs >= 257 and summ.batches < summ.segments
        for i in pick:
            assert out[i][1] == oracle.stats_line(wins[i][0], wins[i][1], oracle.SIEVE), wins[i]
        for i in random.Random(9).sample(range(len(wins) - 1), 16):
            assert out[i][1] == c.verify_range(*wins[i])[1], wins[i]


def test_slice_seeded_segments_config_c3():
    """Three seeded segments of the full 5e13 slice [4e18, 4e18 + 5e13]
    (random.Random(3), the segments bench.py --slice checks), each in a run
    of three consecutive segments under the tuned knobs of the batched form
    (tile-binned hit lists through the prime-multiplier table): the run's
    stats_ref line (every p(n), primes, twins, gaps) and each segment's
    class-map hash against the oracle's exact sieve."""
    import autotune
    a = 4 * 10**18
    b = a + 5 * 10**13
    segs = gbc.segments_of(a, b, gbc.DEFAULT_SEGMENT)
    pick = sorted(random.Random(3).sample(range(len(segs)), 3))
    knobs = autotune.load(autotune.DEFAULT_RECORD)
    with gbc.Context(limit=b, segment_even=gbc.DEFAULT_SEGMENT, hl_mode=1, **knobs) as c:
        for i in pick:
            run = segs[max(0, i - 1):i + 2]
            s, e = run[0][0], run[-1][1]
            c.enqueue_batch(0, run, e)
            res, _ = c.collect(0, len(run))
            assert c.stats().p_hl > 0
            for r in res:
                assert (r.map_hash, r.map_primes) == oracle.map_hash(r.hash_lo, r.hash_hi), (r.seg_start, r.seg_end)
            assert c.verify_range(s, e)[1] == oracle.stats_line(s, e, oracle.SIEVE), (i, s, e)


def test_journaled_slices_resume_and_stop(tmp_path):
    """The slice runner: PASS rows per slice, a stop file ends the run with
    the resume point intact, a second call resumes after the PASS chain;
    each slice's counts equal the oracle's for that slice."""
    a, b, w = 10**12, 10**12 + 8_000_000 - 2, 2_000_000
    j, stop = tmp_path / "journal.txt", tmp_path / "stop"
    with gbc.Context(limit=b, segment_even=1_000_000, max_batch=4) as c:
        assert c.run_slices(a, a + 2 * w - 2, w, j) == (2, False)
        stop.write_text("")
        assert c.run_slices(a, b, w, j, stop_file=stop) == (0, True)
        stop.unlink()
        assert gbc.journal_resume(j, a) == a + 2 * w
        assert c.run_slices(a, b, w, j, stop_file=stop) == (2, False)
    rows = [r.split() for r in j.read_text().splitlines()]
    assert [r[0] for r in rows] == ["PASS"] * 4
    assert [(int(r[1]), int(r[2])) for r in rows] == [(a + i * w, a + i * w + w - 2) for i in range(4)]
    for r in rows:
        got = dict(t.split("=", 1) for t in r[4:] if "=" in t)
        want = dict(t.split("=", 1) for t in oracle.stats_line(int(r[1]), int(r[2]), oracle.SIEVE).split())
        assert got["result"] == "PASS" and got["release"] == "gb300-1.0"
        assert (got["primes"], got["twins"], got["stats_pmax"]) == (want["primes"], want["twins"], want["pmax"])


def test_run_outputs_ridges_live_records(tmp_path):
    """A run's ridge store, live snapshot and records file: the top 30
    ridges, the totals and the largest p(n) equal the oracle's; no record
    events at 1e15."""
    import json
    a, count = 10**15, 2_000_000
    b = a + 2 * (count - 1)
    st, live, rec = tmp_path / "ridges.csv", tmp_path / "live.json", tmp_path / "records.txt"
    with gbc.Context(limit=b, segment_even=1_000_000, max_batch=4, ridge_min=1000) as c:
        c.set_outputs(st, rec, live)
        res, _, _ = c.verify_range(a, b)
    pn = list(oracle.pn_range(a, count))
    want = sorted(((a + 2 * i, p) for i, p in enumerate(pn) if p >= 1000), key=lambda e: (-e[1], -e[0]))[:30]
    got = [tuple(int(x) for x in ln.split(",")[1:3]) for ln in st.read_text().splitlines()
           if ln and not ln.startswith("#")]
    assert got == want
    j = json.loads(live.read_text())
    assert (j["start"], j["limit"], j["evens_done"], j["evens_total"]) == (a, b, count, count)
    assert (j["primes"], j["twins"]) == (res.primes, res.twins)
    assert (j["pmax"], j["pmax_n"]) == (max(pn), a + 2 * pn.index(max(pn)))
    assert j["events"] == [] and (not rec.exists() or rec.read_text() == "")


def test_hitlist_overflow_path_bit_exact():
    """Hit-list bins at 80% of their sizing: marks beyond a region quota or a
    tile bin's capacity take the overflow list (cleared after the tiles); the
    maps (self-check against the rebuild without hit lists) and every
    statistic equal those of the bins at full size."""
    seg = 467_500_000
    a = 4000008233142500000
    segs = [(a, a + seg - 2), (a + seg, a + 2 * seg - 2)]
    limit = segs[-1][1]
    flags = [0, gbc.SEG_VERIFY]
    out = {}
    for pct in (100, 80):
        with gbc.Context(limit=limit, segment_even=seg, max_batch=2, p_mid=1 << 21, mtab_max_gb=96, hl_mode=1,
                         hl_cap_pct=pct, selfcheck_every=1) as c:
            c.enqueue_batch(0, segs, limit, flags)
            res, _ = c.collect(0, 2)
            st = c.stats()
            assert st.selfchecks >= 1
            out[pct] = (res, st.hl_overflow)
    assert out[100][1] == 0 and out[80][1] > 0  # the overflow list was used at 80%
    for r1, r2 in zip(out[100][0], out[80][0]):
        for f in ("primes30", "twins", "ghist"):
            assert list(getattr(r1, f)) == list(getattr(r2, f)), f
        for f in ("map_hash", "map_primes", "gmax_key", "first_prime", "last_prime", "nleft", "pending", "npend",
                  "ntail", "nridge"):
            assert getattr(r1, f) == getattr(r2, f), f
        assert [list(h) for h in r1.hist] == [list(h) for h in r2.hist]
        assert list(r1.first) == list(r2.first)
        assert sorted(zip(r1.tail_g[:r1.ntail], r1.tail_lo[:r1.ntail])) == \
            sorted(zip(r2.tail_g[:r2.ntail], r2.tail_lo[:r2.ntail]))


@pytest.mark.parametrize("plan,first", [(8, 8), (6, 1), (32, 3), (16, 2)])
def test_verify_plan_knobs_same_statistics(plan, first):
    """The verify plan's funnel count and how many funnels every word takes
    before the unresolved words are gathered change only which evens reach
    the exact continuation: primes, twins, gaps, the map hash and the p(n) >=
    3000 tail (counts and first occurrences) stay those of the default plan."""
    seg = 467_500_000
    a = 4000008233142500000
    segs = [(a, a + seg - 2), (a + seg, a + 2 * seg - 2)]
    limit = segs[-1][1]
    flags = [gbc.SEG_VERIFY, gbc.SEG_VERIFY]
    out = []
    for pf, vf in ((0, 0), (plan, first)):
        with gbc.Context(limit=limit, segment_even=seg, max_batch=2, p_mid=1 << 21, mtab_max_gb=96, hl_mode=1,
                         plan_funnels=pf, verify_funnels=vf) as c:
            c.enqueue_batch(0, segs, limit, flags)
            res, _ = c.collect(0, 2)
            out.append(res)
    cand = gbc.candidates()
    tail = [i for i, p in enumerate(cand) if p >= 3000]
    for r1, r2 in zip(*out):
        for f in ("primes30", "twins", "ghist"):
            assert list(getattr(r1, f)) == list(getattr(r2, f)), f
        for f in ("map_hash", "map_primes", "gmax_key", "nleft"):
            assert getattr(r1, f) == getattr(r2, f), f
        assert [sum(r1.hist[cr][i] for cr in range(15)) for i in tail] == \
            [sum(r2.hist[cr][i] for cr in range(15)) for i in tail]
        assert [r1.first[i] for i in tail] == [r2.first[i] for i in tail]


def test_windows_without_sampling_equal_alone_and_the_sampled_run():
    """sample_every = GBC_SAMPLE_NONE: every segment takes the funnel verify +
    exact tail. The windows in shared batches give the same line as alone;
    against the same windows with p(n) of every even, the prime and twin
    counts are equal, and the largest p(n) too wherever it reaches the exact
    tail's bound (else it is reported as 0)."""
    wins = uneven_windows()[:24]
    limit = max(b for _, b in wins)
    kw = dict(limit=limit, segment_even=gbc.DEFAULT_SEGMENT, max_batch=16, max_runs=16, nslots=3)
    with gbc.Context(sample_every=gbc.SAMPLE_NONE, **kw) as c:
        out, summ = c.verify_windows(wins)
        assert summ.batches < summ.segments
        for i in random.Random(10).sample(range(len(wins)), 6):
            assert out[i][1] == c.verify_range(*wins[i])[1], wins[i]
    with gbc.Context(**kw) as c:
        full, _ = c.verify_windows(wins)
    for (a, b), (r, _), (f, _) in zip(wins, out, full):
        assert (r.primes, r.twins, r.evens) == (f.primes, f.twins, f.evens), (a, b)
        assert r.pmax == (f.pmax if f.pmax >= gbc.TAIL_T else 0), (a, b, r.pmax, f.pmax)


def test_runs_hitlist_overflow_selfcheck():
    """Three hit-listed runs in one batch, their marks binned through one
    virtual tile-bin array, with the bins at 80% of their sizing: marks take
    the overflow list, which finds each mark's run; the self-check (the
    rebuild without hit lists, word for word) passes, and every statistic
    equals that of the bins at full size."""
    seg = 467_500_000
    segs, limits = [], []
    for h in (10**16, 10**17, 10**18):
        segs += [(h, h + seg - 2), (h + seg, h + 2 * seg - 2)]
        limits += [h + 2 * seg - 2] * 2
    limit = max(limits)
    flags = [0, gbc.SEG_VERIFY] * 3
    out = {}
    for pct in (100, 80):
        with gbc.Context(limit=limit, segment_even=seg, max_batch=6, max_runs=3, p_mid=1 << 21, mtab_max_gb=96,
                         hl_mode=1, hl_cap_pct=pct, selfcheck_every=1) as c:
            c.enqueue_segments(0, segs, limits, flags)
            res, t = c.collect(0, len(segs))
            assert t.runs == 3
            st = c.stats()
            assert st.selfchecks >= 1
            out[pct] = (res, st.hl_overflow)
    assert out[100][1] == 0 and out[80][1] > 0  # the overflow list was used at 80%
    for r1, r2 in zip(out[100][0], out[80][0]):
        assert result_fields(r1) == result_fields(r2)


def test_uneven_windows_in_64_run_batches_against_oracle():
    """The windows leg's batch shape and knobs (up to 64 segments in up to 64
    runs, their hit lists binned through one virtual tile-bin array, the
    tuned tile and split): 48 uneven
    windows in shared batches; 4 of them (under 2e7 wide) against the
    oracle's exact sieve, 8 against their runs alone."""
    wins = uneven_windows()[:48]
    small = [i for i, (a, b) in enumerate(wins) if b - a < 2 * 10**7]
    pick = random.Random(12).sample(small, 4)
    limit = max(b for _, b in wins)
    with gbc.Context(limit=limit, segment_even=gbc.DEFAULT_SEGMENT, max_batch=64, max_runs=64, nslots=3,
                     tile_bits=1835008, p_mid=1703936, mtab_max_gb=96) as c:
        out, summ = c.verify_windows(wins)
        assert summ.batches < summ.runs  # several runs per batch
        for i in pick:
            assert out[i][1] == oracle.stats_line(wins[i][0], wins[i][1], oracle.SIEVE), wins[i]
        for i in random.Random(13).sample(range(len(wins)), 8):
            assert out[i][1] == c.verify_range(*wins[i])[1], wins[i]
