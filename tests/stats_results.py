"""Per-segment results of the GPU path, restated on the CPU from the oracle
(test infrastructure): the gbc_segment_result fields the run statistics read,
for small windows, so the campaign statistics (gbc_stats_commit) can be
tested without a GPU.

Conventions of the GPU path (gbc_api.cu plan_batch): segment [s, e] of a run
[start, limit] counts the primes q in [s + 1, e + 1] ([s + 1, limit - 1] for
the run's last segment) and the twins (q, q + 2) with q from s + 1 up to
min(that bound, limit - 3); a gap belongs to the segment of its upper prime
and is listed with its lower prime. A sampled segment holds p(n) of every
even; another holds p(n) of the evens the funnel verify left pending, which
here are exactly the evens with p(n) >= 3000 (every one of them is pending on
the GPU).
"""
import numpy as np

import gbc
import oracle

U30 = (1, 7, 11, 13, 17, 19, 23, 29)
TAIL_T = 3000


class PrimeTable:
    """Primality of every odd q in [lo, hi] by the oracle's Miller-Rabin."""

    def __init__(self, lo, hi):
        self.lo = lo | 1
        isp = oracle.lib().gbo_is_prime_u64
        self.bits = np.fromiter((isp(q) for q in range(self.lo, hi + 1, 2)), dtype=np.uint8)

    def primes(self, a, b):
        """The primes in [a, b] (inside the table)."""
        a = max(a | 1, self.lo)
        i0, i1 = (a - self.lo) // 2, (b - self.lo) // 2
        idx = np.nonzero(self.bits[i0:i1 + 1])[0]
        return [self.lo + 2 * int(i0 + i) for i in idx]

    def prev(self, q):
        r = q - 2
        while not self.bits[(r - self.lo) // 2]:
            r -= 2
        return r


def segment_results(start, limit, seg_even, sample_every):
    """gbc_segment_result of every segment of the run [start, limit]
    (gb::plan_segments' segments; segment k sampled when k % sample_every == 0)."""
    cand = gbc.candidates()
    ci = {p: i for i, p in enumerate(cand)}
    segs = gbc.segments_of(start, limit, seg_even)
    tab = PrimeTable(start - 9781 - 4000, limit + 4)
    pn = np.frombuffer(oracle.pn_range(start, (limit - start) // 2 + 1, oracle.SIEVE), dtype=np.uint16)
    out = []
    for k, (s, e) in enumerate(segs):
        r = gbc.SegmentResult()
        last = e == limit
        r.seg_start, r.seg_end, r.evens = s, e, (e - s) // 2 + 1
        r.cnt_lo, r.cnt_hi = s + 1, (limit - 1 if last else e + 1)
        r.twin_hi = min(r.cnt_hi, limit - 3)
        r.hash_lo, r.hash_hi = s - 9781, e + 3
        sampled = k % sample_every == 0
        r.sampled = 1 if sampled else 0
        for c in range(len(cand)):
            r.first[c] = 0xFFFFFFFF
        pend = 0
        for j in range(r.evens):
            n = s + 2 * j
            p = int(pn[(n - start) // 2])
            if not sampled and p < TAIL_T:
                continue
            pend += 1
            i = ci[p]
            r.hist[(n % 30) // 2][i] += 1
            if r.first[i] == 0xFFFFFFFF:
                r.first[i] = j
        if not sampled:
            r.pending = pend
        qs = tab.primes(r.cnt_lo, r.cnt_hi)
        for q in qs:
            r.primes30[U30.index(q % 30)] += 1
        pset = set(tab.primes(r.cnt_lo, r.twin_hi + 2))
        for q in qs:
            if q <= r.twin_hi and q + 2 in pset and q % 30 in (11, 17, 29):
                r.twins[(11, 17, 29).index(q % 30)] += 1
        if qs:
            r.first_prime, r.last_prime = qs[0], qs[-1]
        best = 0
        prev = tab.prev(qs[0]) if qs else 0
        for q in qs:
            g = q - prev
            r.ghist[g // 2] += 1
            best = max(best, (g << 32) | (0xFFFFFFFF - (prev - r.hash_lo)))
            if g >= 700:
                r.tail_g[r.ntail] = g
                r.tail_lo[r.ntail] = prev
                r.ntail += 1
            prev = q
        r.gmax_key = best
        out.append(r)
    return out
