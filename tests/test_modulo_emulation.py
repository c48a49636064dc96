"""The division-free modulo of the sieve kernels (mod_below in
goldbach-l0_gb300/csrc/k_sieve.cu), restated step by step in exact float32
arithmetic (round-toward-zero integer conversions, fused multiply-add and
products rounded to nearest even) and checked against x % p over the
whole precondition x < p * 2^32, 3 <= p < 2^32, including small primes
whose remainder estimate is often negative. A CPU test of the algorithm,
not of the compiled kernel (the GPU tests check that through every map bit).
"""
import math
import random
from fractions import Fraction as F


def rn32(v):
    """v rounded to the nearest float32 (ties to even), as a Fraction."""
    if v == 0:
        return F(0)
    s = -1 if v < 0 else 1
    a = abs(v)
    e = math.floor(math.log2(a))
    while F(2) ** e > a:
        e -= 1
    while F(2) ** (e + 1) <= a:
        e += 1
    ulp = F(2) ** (e - 23)
    q = a / ulp
    n = math.floor(q)
    rem = q - n
    if rem > F(1, 2) or (rem == F(1, 2) and n % 2 == 1):
        n += 1
    return s * n * ulp


def u2f_rz(u):
    if u == 0:
        return F(0)
    e = u.bit_length()
    return F(u) if e <= 24 else F((u >> (e - 24)) << (e - 24))


def f2u_rz(f):
    return min(max(math.floor(f) if f >= 0 else 0, 0), 2**32 - 1)


def f2i_rn(f):
    n = math.floor(f)
    rem = f - n
    if rem > F(1, 2) or (rem == F(1, 2) and n % 2 == 1):
        n += 1
    return n


def mod_below(x, p):
    rp = rn32(F(1, p))
    xf = rn32(u2f_rz(x >> 32) * 2**32 + u2f_rz(x & 0xFFFFFFFF))
    qe = f2u_rz(rn32(xf * rp))
    r = x - qe * p  # exact: |r| < 2^43
    m = abs(r)
    mf = rn32(u2f_rz(m >> 32) * 2**32 + u2f_rz(m & 0xFFFFFFFF))
    rf = -mf if r < 0 else mf
    r -= f2i_rn(rn32(rf * rp)) * p
    if r < 0:
        r += p
    if r >= p:
        r -= p
    return r


def test_mod_below_small_and_large_primes():
    rnd = random.Random(5)
    small = [p for p in range(3, 700) if all(p % d for d in range(2, int(p**0.5) + 1))]
    large = [4194301, 16777213, 1000000007, 2147483647, 3000000019, 4294967291]
    for p in small + large:
        for _ in range(12):
            k = rnd.random()
            if k < 0.3:
                x = rnd.randrange(p * p)
            elif k < 0.6:
                x = rnd.randrange(p << 32)
            else:
                x = (p << 32) - 1 - rnd.randrange(min(p << 32, 1 << 36))
            assert mod_below(x, p) == x % p, (x, p)
