"""The allocation-free class-map entry point (gbc_class_map_noalloc).

It serves callers that cannot call cudaMalloc: code inside another
framework's memory pool with a fixed device budget, and latency-critical
paths that cannot take cudaMalloc's device-wide synchronization. It builds
the class map of a q range in a buffer the caller owns and keeps its scratch
in a fixed device array of the library. Here the test is that caller: it owns
the primes and the map buffers (allocated with torch), calls the entry point
twice in a row on two different windows, and compares each map bit for bit
with the map the per-segment path (gbc_enqueue_batch) built for the same q
range, checks it against the oracle's hash of the primes in the range, and
checks that every bit past the range is zero. The file is named so pytest
collects it last: a failure here stops a -x run only after every other test
has run. A third test records the call inside a CUDA graph capture and replays
it. The argument checks run on the host before any CUDA call, so they are
tested without a GPU.
"""
import ctypes as C

import numpy as np
import pytest

import gbc
import oracle

U30 = (1, 7, 11, 13, 17, 19, 23, 29)


def odd_primes_upto(n):
    s = np.ones(n + 1, dtype=bool)
    s[:2] = False
    for i in range(2, int(n ** 0.5) + 1):
        if s[i]:
            s[i * i::i] = False
    p = np.nonzero(s)[0]
    return p[p > 2].astype(np.uint32)


def existing_map(a, b, seg):
    """The class map the per-segment contract builds for evens [a, b]."""
    segs = gbc.segments_of(a, b, seg)
    with gbc.Context(limit=b, segment_even=seg, max_batch=len(segs)) as c:
        c.enqueue_batch(0, segs, b)
        c.collect(0, len(segs))
        base, nblk, wpc, words = c.map(0)
    return base, nblk, wpc, np.frombuffer(words, dtype=np.uint32).copy()


def class_bits(words, wpc, nbits):
    w = words.reshape(8, -1)[:, :wpc]
    bits = np.unpackbits(np.ascontiguousarray(w).view(np.uint8), axis=1, bitorder="little")
    return bits[:, :nbits]


def splitmix64(q):
    with np.errstate(over="ignore"):
        z = q + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def map_hash(bits, base):
    """Sum mod 2^64 of splitmix64(q) over the set bits, and their count (the
    oracle's class-map hash, gbo_map_hash)."""
    h, c = np.uint64(0), 0
    for k in range(8):
        t = np.nonzero(bits[k])[0].astype(np.uint64)
        q = np.uint64(base) + np.uint64(30) * t + np.uint64(U30[k])
        with np.errstate(over="ignore"):
            h = h + np.sum(splitmix64(q), dtype=np.uint64)
        c += len(t)
    return int(h), c


def noalloc_map(lib, torch, q_lo, q_hi, primes_dev, nprimes, max_prime, stream):
    base, nblk, wpc = C.c_uint64(), C.c_uint32(), C.c_uint32()
    err = C.create_string_buffer(256)
    # sizing call: returns the layout and GBC_E_ARG without launching anything
    rc = lib.gbc_class_map_noalloc(q_lo, q_hi, primes_dev, nprimes, max_prime, None, 0, C.byref(base),
                                   C.byref(nblk), C.byref(wpc), stream, err, len(err))
    assert rc == -1 and wpc.value > 0
    # filled with ones first: every word past the range must come back zero
    out = torch.full((8 * wpc.value,), -1, dtype=torch.int32, device="cuda")
    rc = lib.gbc_class_map_noalloc(q_lo, q_hi, primes_dev, nprimes, max_prime, C.c_void_p(out.data_ptr()),
                                   8 * wpc.value, C.byref(base), C.byref(nblk), C.byref(wpc), stream, err,
                                   len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    return base.value, nblk.value, wpc.value, out.cpu().numpy().view(np.uint32)


@pytest.mark.gpu
def test_noalloc_map_matches_existing_path_twice():
    torch = pytest.importorskip("torch")
    lib = gbc.load()
    primes = odd_primes_upto(1_650_000)
    assert len(primes) <= 131072  # GBC_NOALLOC_MAX_PRIMES
    pd = torch.from_numpy(primes.view(np.int32)).to("cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    windows = [(10**12, 10**12 + 3_999_998, 1_000_000), (2_500_000_000_000, 2_500_000_000_000 + 5_999_998, 2_000_000)]
    for a, b, seg in windows:  # two calls in a row, different windows
        base, nblk, wpc, words = existing_map(a, b, seg)
        q_hi = base + 30 * (nblk - 1) + 29
        nb, nn, nw, got = noalloc_map(lib, torch, base, q_hi, C.c_void_p(pd.data_ptr()), len(primes),
                                      int(primes[-1]), stream)
        assert (nb, nn) == (base, nblk)
        mine = class_bits(got, nw, nblk)
        assert np.array_equal(mine, class_bits(words, wpc, nblk))
        assert map_hash(mine, base) == oracle.map_hash(base, q_hi)
        assert not class_bits(got, nw, 32 * nw)[:, nblk:].any(), "bits past the range must be zero"


@pytest.mark.gpu
def test_noalloc_map_inside_a_captured_graph():
    """The use the entry point exists for: the call recorded while the
    caller's stream is being captured (torch.cuda.graph), after one warm
    call outside the capture; replaying the graph writes the same map as
    the per-segment path, with every bit past the range zero."""
    torch = pytest.importorskip("torch")
    lib = gbc.load()
    primes = odd_primes_upto(1_650_000)
    pd = torch.from_numpy(primes.view(np.int32)).to("cuda")
    a, b, seg = 2 * 10**12, 2 * 10**12 + 3_999_998, 1_000_000  # primes to 1.65e6 reach sqrt(b)
    base, nblk, wpc, words = existing_map(a, b, seg)
    q_hi = base + 30 * (nblk - 1) + 29
    warm = noalloc_map(lib, torch, base, q_hi, C.c_void_p(pd.data_ptr()), len(primes), int(primes[-1]),
                       C.c_void_p(torch.cuda.current_stream().cuda_stream))
    nw = warm[2]
    out = torch.full((8 * nw,), -1, dtype=torch.int32, device="cuda")
    b_out, n_out, w_out = C.c_uint64(), C.c_uint32(), C.c_uint32()
    err = C.create_string_buffer(256)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = lib.gbc_class_map_noalloc(base, q_hi, C.c_void_p(pd.data_ptr()), len(primes), int(primes[-1]),
                                       C.c_void_p(out.data_ptr()), 8 * nw, C.byref(b_out), C.byref(n_out),
                                       C.byref(w_out), C.c_void_p(torch.cuda.current_stream().cuda_stream), err,
                                       len(err))
    assert rc == 0, err.value.decode()
    out.fill_(-1)  # the replay, not the capture, must write the map
    g.replay()
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    assert (b_out.value, n_out.value) == (base, nblk)
    assert np.array_equal(class_bits(got, nw, nblk), class_bits(words, wpc, nblk))
    assert not class_bits(got, nw, 32 * nw)[:, nblk:].any(), "bits past the range must be zero"


def test_noalloc_rejects_sizes_beyond_its_limits():
    lib = gbc.load()
    err = C.create_string_buffer(256)
    dummy = C.c_void_p(1)
    rc = lib.gbc_class_map_noalloc(10**12, 10**12 + 2**31, dummy, 1000, 1_500_000, None, 0, None, None, None,
                                   None, err, len(err))
    assert rc == -1 and b"GBC_NOALLOC_MAX_SPAN" in err.value
    rc = lib.gbc_class_map_noalloc(10**12, 10**12 + 1000, dummy, 200_000, 2_750_000, None, 0, None, None, None,
                                   None, err, len(err))
    assert rc == -1 and b"GBC_NOALLOC_MAX_PRIMES" in err.value
    # 999 odd primes end at 7919, whose square is below the range
    rc = lib.gbc_class_map_noalloc(10**12, 10**12 + 1000, dummy, 999, 7919, None, 0, None, None, None, None, err,
                                   len(err))
    assert rc == -1 and b"sqrt" in err.value
    # a list that does not start at 3 (or misses a prime) has the wrong count
    rc = lib.gbc_class_map_noalloc(10**6, 10**6 + 1000, dummy, 1000, 7919, None, 0, None, None, None, None, err,
                                   len(err))
    assert rc == -1 and b"every odd prime from 3" in err.value
