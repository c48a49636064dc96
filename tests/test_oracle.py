"""The CPU oracle against the reference's golden data (no GPU).

Pins oracle/gb_oracle.c to: the output of the reference's own stats_ref
(tests/stats_ref.cpp) on ten windows, p(n) from the reference's
cpu_min_goldbach_prime (src/primes.cpp:482-493) on four windows and four
digests, the published S(p) table of tests/stats_ref.cpp:35-42 and the
base-2 pseudoprimes below 2^32 of tests/data/psp2_below_2_32.txt, the same
checks the reference's host_tests and stats_ref --known make.
"""
import hashlib
import struct

import pytest

import oracle
from conftest import golden_path, known_sp, pn_digests, pn_fixture, stats_windows


def test_psp2_below_2_32_are_composite():
    lib = oracle.lib()
    with open(golden_path("psp2_below_2_32.txt")) as f:
        nums = [int(x) for x in f]
    assert len(nums) == 10403
    assert not any(lib.gbo_is_prime_u64(n) for n in nums)


def test_mr_small_primes_exact():
    # trial division against Miller-Rabin below 10^5, and the 2^64 edge
    def td(n):
        if n < 2:
            return False
        d = 2
        while d * d <= n:
            if n % d == 0:
                return False
            d += 1
        return True
    assert all(oracle.is_prime(n) == td(n) for n in range(0, 100000))
    assert oracle.is_prime(18446744073709551557)          # largest prime below 2^64
    assert not oracle.is_prime(18446744073709551615)
    assert not oracle.is_prime(3825123056546413051)       # strong psp to bases 2..23


@pytest.mark.parametrize("p,S,rec", known_sp())
def test_known_sp_table(p, S, rec):
    assert oracle.min_goldbach_prime(S) == p
    if rec:
        lo = max(6, S - 4000) if S > 4002 else 6
        pn = oracle.pn_range(lo, (S - lo) // 2, oracle.MR)
        assert max(pn) < p


@pytest.mark.parametrize("start,limit,line", stats_windows(), ids=lambda x: str(x)[:12])
def test_stats_sieve_mode_matches_stats_ref(start, limit, line):
    assert oracle.stats_line(start, limit, oracle.SIEVE) == line


@pytest.mark.parametrize("idx", [0, 7])
def test_stats_mr_mode_matches_stats_ref(idx):
    start, limit, line = stats_windows()[idx]
    assert oracle.stats_line(start, limit, oracle.MR) == line


@pytest.mark.parametrize("tag", ["low", "1e12", "4e18", "top"])
@pytest.mark.parametrize("mode", [oracle.MR, oracle.SIEVE])
def test_pn_windows(tag, mode):
    ns, ps = pn_fixture(tag)
    got = oracle.pn_range(ns[0], len(ns), mode)
    assert list(got) == ps


@pytest.mark.parametrize("start,count,digest", pn_digests())
def test_pn_digests(start, count, digest):
    got = oracle.pn_range(start, count, oracle.SIEVE)
    assert hashlib.sha256(struct.pack(f"<{count}H", *got)).hexdigest() == digest


def test_map_hash_definition():
    # the hash is the sum of splitmix64 over the primes coprime to 30
    a, b = 4000000000000000000, 4000000000000100000
    h, c = oracle.map_hash(a, b)
    hh, cc = 0, 0
    for q in range(a | 1, b + 1, 2):
        if q % 3 and q % 5 and oracle.is_prime(q):
            hh = (hh + oracle.lib().gbo_mix(q)) % (1 << 64)
            cc += 1
    assert (h, c) == (hh, cc)
