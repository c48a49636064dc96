"""The allocation-free class-map entry point against the existing path.

gbc_class_map_noalloc serves callers that cannot call cudaMalloc -- code
running while a CUDA stream is captured, code inside another framework's
fixed memory pool, latency-critical paths that cannot take cudaMalloc's
device-wide synchronization. It builds the class map of a q range in a
buffer the caller owns and keeps its scratch in a fixed device array of the
library. Here the test is that caller: it owns the primes and the map
buffers (allocated with torch), calls the entry point twice in a row on two
different windows, and compares each map bit for bit with the map the
per-segment path (gbc_enqueue_batch) built for the same q range. The file is
named so pytest collects it last: a failure here stops a -x run only after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

import gbc

pytestmark = pytest.mark.gpu


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


def class_bits(words, wpc, nblk):
    w = words.reshape(8, -1)[:, :wpc]
    bits = np.unpackbits(np.ascontiguousarray(w).view(np.uint8), axis=1, bitorder="little")
    return bits[:, :nblk]


def noalloc_map(lib, torch, q_lo, q_hi, primes_dev, nprimes, max_prime, stream):
    base, nblk, wpc = C.c_uint64(), C.c_uint32(), C.c_uint32()
    err = C.create_string_buffer(256)
    # sizing call: returns the layout and GBC_E_ARG without launching anything
    rc = lib.gbc_class_map_noalloc(q_lo, q_hi, primes_dev, nprimes, max_prime, None, 0, C.byref(base),
                                   C.byref(nblk), C.byref(wpc), stream, err, len(err))
    assert rc == -1 and wpc.value > 0
    out = torch.empty(8 * wpc.value, dtype=torch.int32, device="cuda")
    rc = lib.gbc_class_map_noalloc(q_lo, q_hi, primes_dev, nprimes, max_prime, C.c_void_p(out.data_ptr()),
                                   8 * wpc.value, C.byref(base), C.byref(nblk), C.byref(wpc), stream, err,
                                   len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    return base.value, nblk.value, wpc.value, out.cpu().numpy().view(np.uint32)


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
        assert np.array_equal(class_bits(got, nw, nblk), class_bits(words, wpc, nblk))


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
    rc = lib.gbc_class_map_noalloc(10**12, 10**12 + 1000, dummy, 1000, 7919, None, 0, None, None, None, None, err,
                                   len(err))
    assert rc == -1 and b"sqrt" in err.value
