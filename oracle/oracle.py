"""ctypes access to the CPU oracle (oracle/gb_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py to verify results or as the timed CPU baseline, never
by the GPU product path.
"""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.gbo_is_prime_u64.restype = C.c_int
        L.gbo_is_prime_u64.argtypes = [C.c_uint64]
        L.gbo_min_goldbach_prime.restype = C.c_uint64
        L.gbo_min_goldbach_prime.argtypes = [C.c_uint64]
        L.gbo_stats_line.restype = C.c_int
        L.gbo_stats_line.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_char_p, C.c_size_t]
        L.gbo_pn_range.restype = C.c_int
        L.gbo_pn_range.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.POINTER(C.c_uint16)]
        L.gbo_map_hash.restype = C.c_int
        L.gbo_map_hash.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.gbo_mix.restype = C.c_uint64
        L.gbo_mix.argtypes = [C.c_uint64]
        _lib = L
    return _lib


MR, SIEVE = 0, 1


def is_prime(n):
    return bool(lib().gbo_is_prime_u64(n))


def min_goldbach_prime(n):
    return lib().gbo_min_goldbach_prime(n)


def stats_line(start, limit, mode=SIEVE, threads=0):
    buf = C.create_string_buffer(1 << 20)
    rc = lib().gbo_stats_line(start, limit, mode, threads, buf, len(buf))
    if rc:
        raise RuntimeError(f"oracle stats failed ({rc}) for [{start}, {limit}]")
    return buf.value.decode()


def pn_range(start, count, mode=SIEVE, threads=0):
    out = (C.c_uint16 * count)()
    rc = lib().gbo_pn_range(start, count, mode, threads, out)
    if rc:
        raise RuntimeError(f"oracle p(n) failed ({rc})")
    return out


def map_hash(a, b, threads=0):
    h, c = C.c_uint64(), C.c_uint64()
    lib().gbo_map_hash(a, b, threads, C.byref(h), C.byref(c))
    return h.value, c.value
