"""CPU oracle of the sparse class map (the reference's --sparse path:
include/sparse.hpp:1-33 geometry, src/sparse.cpp, kernels/sparse.cl).

TEST INFRASTRUCTURE ONLY: used by tests/ to verify results, never by the GPU
product path.

The reference validates its sparse path against an independent CPU sieve of
the same class progressions and Miller-Rabin spot checks (its debug_sparse
tool, docs/HISTORY.md section 9.2k "Validation"), and its host tests check
that the residues are sorted units reaching every even class and that a
first hit is the first multiple in its class (tests/host_tests.cpp:473-530).
This module restates those checks:
  class_map   bit t of class k <-> q = N - M TB + c_k + M t is prime, by a
              sieve of each progression with t0 = -(Q + c_k) * M^-1 mod l
              (Fermat inverse), a different derivation from the product's
              first-hit formula
  map_by_mr   the same bits by Miller-Rabin on every q (any height)
  usable / cover_ok / candidates: the residue and candidate rules
  first_witness: the first candidate in a given order with n - p prime
Parity is pinned to the mathematics (primality by deterministic
Miller-Rabin), not to reference outputs: the reference's sparse path is GPU
code (Level Zero) that does not run here.
"""
import math

import numpy as np

import oracle

M = 30030


def usable(r, res):
    """Classes k whose candidates p = r - c_k (mod M) can be prime."""
    return [k for k, c in enumerate(res) if math.gcd((r - c) % M, M) == 1]


def cover_ok(res):
    return all(usable(r, res) for r in range(0, M, 2))


def primes_upto(n):
    s = np.ones(n + 1, dtype=bool)
    s[:2] = False
    s[4::2] = False
    for p in range(3, math.isqrt(n) + 1, 2):
        if s[p]:
            s[p * p::2 * p] = False
    return np.nonzero(s)[0]


def candidates(r, res, pmax, isp=None):
    """Every candidate p <= pmax of even class r: the primes of the usable
    classes' residues r - c_k (mod M), as (p, k) pairs."""
    out = []
    for k in usable(r, res):
        s0 = (r - res[k]) % M
        for p in range(s0, pmax + 1, M):
            if (isp[p] if isp is not None else oracle.is_prime(p)):
                out.append((p, k))
    return out


def _powmod_vec(b, e, m):
    """b^e mod m elementwise, m < 2^32 (products stay below 2^64)."""
    b = b % m
    r = np.ones_like(m)
    e = e.copy()
    while e.any():
        odd = (e & 1).astype(bool)
        r = np.where(odd, (r * b) % m, r)
        b = (b * b) % m
        e >>= 1
    return r


def class_map(n0, dl, tb, res):
    """K bool arrays of dl + tb bits: the exact sparse map of the segment at
    n0 (a multiple of M) by a sieve of each class progression. Needs
    n0 - M tb above sqrt of the largest q (no q is a sieving prime)."""
    T = dl + tb
    Q = n0 - M * tb
    qmax = Q + max(res) + M * (T - 1)
    lim = math.isqrt(qmax) + 1
    assert Q > lim
    ps = primes_upto(lim)
    ps = ps[ps > 13].astype(np.uint64)
    inv = _powmod_vec(np.uint64(M) % ps, ps - np.uint64(2), ps)  # M^-1 mod l (Fermat)
    rows = []
    for c in res:
        row = np.ones(T, dtype=bool)
        # t0 = -(Q + c) * M^-1 mod l, i.e. Q + c + M t0 = 0 (mod l)
        t0 = ((ps - _mod_u64(Q + c, ps)) % ps) * inv % ps
        few = ps <= np.uint64(T)
        for l, t in zip(ps[few].tolist(), t0[few].tolist()):
            row[t::l] = False
        one = ~few & (t0 < np.uint64(T))
        row[t0[one].astype(np.int64)] = False
        rows.append(row)
    return rows


def _mod_u64(x, m):
    """x mod m elementwise for a Python int x < 2^64 and m < 2^32."""
    hi, lo = divmod(x, 1 << 32)
    r = (np.uint64(hi) % m) * np.uint64(1 << 32) % m
    return (r + np.uint64(lo) % m) % m


def map_by_mr(n0, dl, tb, res):
    """The same bits by Miller-Rabin on every q."""
    T = dl + tb
    Q = n0 - M * tb
    return [np.array([oracle.is_prime(Q + c + M * t) for t in range(T)], dtype=bool) for c in res]


def to_words(bits):
    """bool bits -> u32 words, bit b of word w <-> index 32 w + b."""
    n = (len(bits) + 31) // 32 * 32
    b = np.zeros(n, dtype=bool)
    b[: len(bits)] = bits
    return np.packbits(b, bitorder="little").view("<u4").tolist()


def first_witness(n, plan):
    """The first p of plan (a list of p) with n - p prime; 0 if none."""
    for p in plan:
        if oracle.is_prime(n - p):
            return p
    return 0
