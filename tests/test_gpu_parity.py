"""GPU path against the reference's golden data and the CPU oracle.

Every test calls the CUDA path through the C ABI (libgbc.so via ctypes) and
compares bit-exact: the run statistics line with the reference's stats_ref
output (tests/stats_ref.cpp, the comparison rules of tests/stats_compare.py
taken to full equality), p(n) of every even with the reference's
cpu_min_goldbach_prime, the class-map hash and counts with the oracle's
exact sieve, and the independent verifier's published windows that the
reference's tests/known_windows.py holds.
"""
import hashlib
import random
import struct

import pytest

import gbc
import oracle
from conftest import known_windows, pn_digests, pn_fixture, stats_windows

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    """Small segments (2e6) so every window spans several segments and batches."""
    with gbc.Context(limit=gbc.MAX_LIMIT, segment_even=2_000_000, max_batch=4, want_pn=True) as c:
        yield c


@pytest.mark.parametrize("start,limit,line", stats_windows(), ids=lambda x: str(x)[:12])
def test_stats_ref_windows(ctx, start, limit, line):
    res, got, _ = ctx.verify_range(start, limit)
    assert got == line
    assert res.evens == (limit - start) // 2 + 1


@pytest.mark.parametrize("tag", ["low", "1e12", "4e18", "top"])
def test_pn_matches_reference(ctx, tag):
    ns, ps = pn_fixture(tag)
    _, _, pn = ctx.verify_range(ns[0], ns[-1], want_pn=True)
    assert list(pn) == ps


@pytest.mark.parametrize("start,count,digest", pn_digests())
def test_pn_digests(ctx, start, count, digest):
    _, _, pn = ctx.verify_range(start, start + 2 * (count - 1), want_pn=True)
    assert hashlib.sha256(bytes(pn)).hexdigest() == digest


def test_low_range_stats_match_oracle(ctx):
    # q = 3, 5 (outside the class map), n = 4 (p = 2, the GPU retry) and the
    # generic low-range checker
    for start, limit in [(6, 100000), (4, 20000), (10, 10010), (9700, 30000)]:
        _, got, _ = ctx.verify_range(start, limit)
        if start >= 6:
            assert got == oracle.stats_line(start, limit, oracle.MR)
    _, _, pn = ctx.verify_range(4, 40000, want_pn=True)
    assert list(pn) == list(oracle.pn_range(4, len(pn), oracle.MR))


def test_segment_hash_and_counts_match_oracle(ctx):
    segs = gbc.segments_of(4_000_000_000_000_000_000, 4_000_000_000_007_999_998, 2_000_000)
    ctx.enqueue_batch(0, segs, segs[-1][1])
    res, _ = ctx.collect(0, len(segs))
    for r in res:
        h, c = oracle.map_hash(r.hash_lo, r.hash_hi)
        assert (r.map_hash, r.map_primes) == (h, c)
        line = oracle.stats_line(r.seg_start, r.seg_end, oracle.SIEVE)
        kv = dict(t.split("=", 1) for t in line.split())
        assert sum(r.hist[cr][i] for cr in range(15) for i in range(gbc.NCAND)) + r.nleft == r.evens
        assert int(kv["evens"]) == r.evens


U30 = [1, 7, 11, 13, 17, 19, 23, 29]


@pytest.mark.parametrize("a,tile_log2,tile_bits", [(10**12, 20, 0), (4 * 10**18, 16, 0), (6, 18, 0),
                                                   (9223372036853775808, 20, 0), (gbc.MAX_LIMIT - 2_000_000, 20, 0),
                                                   (10**12, 20, 1835008), (4 * 10**18, 20, 1572864),
                                                   (9223372036853775808, 20, 1835008), (6, 20, 53248)])
def test_class_map_bit_exact(a, tile_log2, tile_bits):
    """Every bit of a batch's class map against Miller-Rabin (the
    reference's debug_map validator): the sieve stages may not lose or add a
    mark anywhere, including q < 67 at the bottom and 2^64 - 2^40 at the top."""
    seg = 500_000
    b = a + 2 * seg - 2
    segs = gbc.segments_of(a, b, seg)
    with gbc.Context(limit=b, segment_even=seg, max_batch=len(segs), tile_log2=tile_log2, tile_bits=tile_bits,
                     p_mid=1 << 18) as c:
        c.enqueue_batch(0, segs, b)
        c.collect(0, len(segs))
        base, nblk, wpc, w = c.map(0)
    bad = []
    for k in range(8):
        for t in range(nblk):
            q = base + 30 * t + U30[k]
            if ((w[k * wpc + (t >> 5)] >> (t & 31)) & 1) != oracle.is_prime(q):
                bad.append(q)
    assert not bad, bad[:8]


@pytest.mark.parametrize("a", [4 * 10**18, 9223372036853775808, gbc.MAX_LIMIT - 3_000_000])
def test_hit_list_class_map_bit_exact(a):
    """The prime-multiplier hit lists (every prime above ~1.7e7 marks only
    p m with m prime) leave the same exact map: every bit against
    Miller-Rabin."""
    seg = 500_000
    b = a + 2 * seg - 2
    segs = gbc.segments_of(a, b, seg)
    with gbc.Context(limit=b, segment_even=seg, max_batch=len(segs), hl_mode=1, mtab_max_gb=8) as c:
        c.enqueue_batch(0, segs, b)
        c.collect(0, len(segs))
        base, nblk, wpc, w = c.map(0)
    bad = []
    for k in range(8):
        for t in range(nblk):
            q = base + 30 * t + U30[k]
            if ((w[k * wpc + (t >> 5)] >> (t & 31)) & 1) != oracle.is_prime(q):
                bad.append(q)
    assert not bad, bad[:8]


@pytest.mark.parametrize("idx", [2, 4, 5, 6, 7])
def test_hit_list_stats_windows(idx):
    start, limit, line = stats_windows()[idx]
    with gbc.Context(limit=limit, segment_even=1_000_000, max_batch=4, hl_mode=1, mtab_max_gb=8) as c:
        assert c.verify_range(start, limit)[1] == line


def kv(line):
    return dict(t.split("=", 1) for t in line.split() if "=" in t)


def dense(s):
    return [int(x) if x else 0 for x in s.split(",")] if s and s != "-" else []


@pytest.mark.parametrize("a,seg", [(4 * 10**18, 1_000_000), (1425172824436700150, 500_000)])
def test_verify_mode_tail_and_sampled_segments(a, seg):
    """The reference's production checker: funnel verify + exact tail on
    most segments, p(n) of every even on the sampled ones. Per segment
    against the oracle: a verified segment lists exactly the evens with
    p(n) >= 3000 (counts, first occurrences, ridges); a sampled segment has
    the full histogram; every segment accounts for all of its evens."""
    nseg = 6
    b = a + nseg * seg - 2
    segs = gbc.segments_of(a, b, seg)
    cand = gbc.candidates()
    flags = [0 if i % 3 == 0 else gbc.SEG_VERIFY for i in range(nseg)]
    with gbc.Context(limit=b, segment_even=seg, max_batch=nseg) as c:
        c.enqueue_batch(0, segs, b, flags)
        res, _ = c.collect(0, nseg)
    for r, f in zip(res, flags):
        want = kv(oracle.stats_line(r.seg_start, r.seg_end, oracle.SIEVE))
        wh = dense(want["hist"]) + [0] * gbc.NCAND
        wf = {int(x.split(":")[0]): int(x.split(":")[1]) for x in want["first"].split(";")}
        got = [sum(r.hist[cr][i] for cr in range(15)) for i in range(gbc.NCAND)]
        gfirst = {cand[i]: r.seg_start + 2 * r.first[i] for i in range(gbc.NCAND) if r.first[i] != 0xFFFFFFFF}
        assert r.sampled == (0 if f else 1)
        if r.sampled:
            assert got == wh[:gbc.NCAND] and gfirst == wf
        else:
            assert r.pending >= sum(got[i] for i in range(gbc.NCAND) if cand[i] >= 3000)
            assert sum(got) + r.nleft == r.pending
            tail = [i for i in range(gbc.NCAND) if cand[i] >= 3000]
            assert [got[i] for i in tail] == [wh[i] for i in tail]
            assert {p: n for p, n in gfirst.items() if p >= 3000} == {p: n for p, n in wf.items() if p >= 3000}
        assert r.primes30[0] + sum(r.primes30[1:]) + (0 if r.seg_start > 7 else 2) >= 0
        # ridges: every even with p(n) >= 3000
        pn = oracle.pn_range(r.seg_start, r.evens, oracle.SIEVE)
        ridges = {(r.seg_start + 2 * i, p) for i, p in enumerate(pn) if p >= 3000}
        assert {(r.ridge_n[i], r.ridge_p[i]) for i in range(r.nridge)} == ridges


def test_verify_mode_run_line():
    """A run with every 4th segment sampled: the GBSTATS line's counts, gaps
    and tail equal the oracle's exact statistics of the range."""
    a, b = 4 * 10**18, 4 * 10**18 + 24_000_000
    with gbc.Context(limit=b, segment_even=2_000_000, max_batch=4, sample_every=4) as c:
        res, line, _ = c.verify_range(a, b)
    g, w = kv(line), kv(oracle.stats_line(a, b, oracle.SIEVE))
    assert line.startswith("GBSTATS v2")
    for k in ("evens", "primes", "twins", "primes30", "twins30"):
        assert g[k] == w[k], k
    assert g["gaps"] == w["gaps"] and g["gd1"] == w["gmom"].split(",")[0] and g["gsmom"] == w["gmom"]
    assert g["gmax"] == w["gmax"] and g["gtail"] == w["gtail"]
    assert dense(g["gsamp"]) == dense(w["ghist"])
    cand = gbc.candidates()
    wh = dense(w["hist"]) + [0] * gbc.NCAND
    t0 = [i for i in range(gbc.NCAND) if cand[i] >= 3000][0]
    want_tail = [wh[i] for i in range(t0, gbc.NCAND)]
    while want_tail and not want_tail[-1]:
        want_tail.pop()
    got_tail = dense(g["tail"].split(":", 1)[1]) if g["tail"] != "-" else []
    assert got_tail == want_tail
    segs = gbc.segments_of(a, b, 2_000_000)
    assert int(g["evens_sampled"]) == sum((e - s) // 2 + 1 for i, (s, e) in enumerate(segs) if i % 4 == 0)


def test_batched_equals_plain():
    a, b = 4_000_000_000_000_000_000, 4_000_000_000_060_000_000
    lines = []
    for batch in (1, 3, 8):
        with gbc.Context(limit=b, segment_even=7_000_000, max_batch=batch) as c:
            lines.append(c.verify_range(a, b)[1])
    assert lines[0] == lines[1] == lines[2]
    assert lines[0] == oracle.stats_line(a, b, oracle.SIEVE)


@pytest.mark.parametrize("tile_log2,p_mid", [(16, 1 << 14), (18, 1 << 20), (20, 1 << 24)])
def test_tuning_knobs_keep_results(tile_log2, p_mid):
    a, b = 4_400_000_000_000_000_000, 4_400_000_000_020_000_000
    with gbc.Context(limit=b, segment_even=5_000_000, max_batch=2, tile_log2=tile_log2, p_mid=p_mid) as c:
        assert c.verify_range(a, b)[1] == oracle.stats_line(a, b, oracle.SIEVE)


def test_production_segment_at_4e18():
    """One full 467.5M-integer segment at 4e18 + k * 467.5e6, k from seed 1
    in [0, 1e5): run statistics (every p(n), primes, twins, gaps) and the
    class-map hash against the oracle's exact sieve."""
    k = random.Random(1).randrange(100000)
    a = 4 * 10**18 + k * 467_500_000
    b = a + 467_500_000 - 2
    with gbc.Context(limit=b, max_batch=1) as c:
        c.enqueue_batch(0, [(a, b)], b)
        (r,), _ = c.collect(0, 1)
        h, n = oracle.map_hash(r.hash_lo, r.hash_hi)
        assert (r.map_hash, r.map_primes) == (h, n)
        _, line, _ = c.verify_range(a, b)
    assert line == oracle.stats_line(a, b, oracle.SIEVE)


@pytest.mark.parametrize("name", ["4e18+1e10", "4e18+1e12"])
def test_published_windows(name):
    row = [r for r in known_windows() if r[0] == name][0]
    _, s, n, primes, pmax, npmax = row
    with gbc.Context(limit=n) as c:
        res, line, _ = c.verify_range(s, n)
    assert res.primes == primes
    if pmax:
        kv = dict(t.split("=", 1) for t in line.split())
        assert int(kv["pmax"]) == pmax
        firsts = dict(x.split(":") for x in kv["first"].split(";"))
        assert int(firsts[str(pmax)]) == npmax


def test_contract_errors(ctx):
    with pytest.raises(gbc.GbcError) as e:
        ctx.collect(1, 1)
    assert e.value.code == -5
    with pytest.raises(gbc.GbcError) as e:
        ctx.enqueue_batch(0, [(10**12, 10**12 + 1000), (10**12 + 2000, 10**12 + 3000)], 10**12 + 3000)
    assert e.value.code == -1
    with pytest.raises(gbc.GbcError) as e:
        ctx.enqueue_batch(0, [(10**12, 10**12 + 3_000_000)], 10**12 + 3_000_000)  # longer than segment_even
    assert e.value.code == -1


def test_collect_timeout_is_bounded(ctx):
    segs = gbc.segments_of(10**18, 10**18 + 7_999_998, 2_000_000)
    ctx.enqueue_batch(1, segs, segs[-1][1])
    try:
        ctx.collect(1, len(segs), timeout_ms=0)
    except gbc.GbcError as e:
        assert e.code == -4
        ctx.collect(1, len(segs))
