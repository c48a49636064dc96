"""The bounded device waits run out and the batch fails closed (GPU).

Each test makes one wait of the pipeline give up through the context's
test_flags (include/gbc.h GBC_TEST_*), with nothing that can fault or hang
the GPU: a wait that gives up sets an error flag and the kernel returns.
gbc_collect must then report GBC_E_DEVICE with the flag, nothing is merged,
and the GPU stays usable: the same batch on a fresh context passes.
"""
import pytest

import gbc
import oracle

pytestmark = pytest.mark.gpu

K_ERR_RETRY = 1 << 4
K_ERR_STAGING = 1 << 9


def flags_of(err):
    return int(str(err).split("device error flags 0x")[1].split()[0], 16)


def test_staging_wait_that_runs_out_fails_closed():
    """The first wait on the bulk copies into shared memory gives up at once
    (the tile bins staged into the tile sieve of a hit-list batch, the chunks
    staged into the verify checker); its second wait lets the copies land."""
    seg = 500_000
    a = 4 * 10**18
    b = a + 4 * seg - 2
    segs = gbc.segments_of(a, b, seg)
    flags = [0] + [gbc.SEG_VERIFY] * (len(segs) - 1)
    kw = dict(limit=b, segment_even=seg, max_batch=len(segs), hl_mode=1, mtab_max_gb=8)
    with gbc.Context(test_flags=gbc.TEST_STAGING_WAIT, **kw) as c:
        c.enqueue_batch(0, segs, b, flags)
        with pytest.raises(gbc.GbcError) as e:
            c.collect(0, len(segs))
        assert e.value.code == -3 and flags_of(e.value) & K_ERR_STAGING
        assert c.stats().p_hl > 0  # a hit-list batch: the tile bins were staged
    with gbc.Context(**kw) as c:
        c.enqueue_batch(0, segs, b, flags)
        res, _ = c.collect(0, len(segs))
        assert all(r.err == 0 for r in res)
        # the same segments through the whole run: the oracle's line
        assert c.verify_range(a, b)[1] == oracle.stats_line(a, b, oracle.SIEVE)


def test_retry_search_that_runs_out_fails_closed():
    """With one candidate per class the exact checker leaves most evens to
    the GPU retry, whose search stops after one try: the retry's flag."""
    a, b = 10**6, 10**6 + 198
    with gbc.Context(limit=b, segment_even=1000, max_batch=1, test_flags=gbc.TEST_RETRY_LIMIT) as c:
        c.enqueue_batch(0, [(a, b)], b)
        with pytest.raises(gbc.GbcError) as e:
            c.collect(0, 1)
        assert e.value.code == -3 and flags_of(e.value) & K_ERR_RETRY
    with gbc.Context(limit=b, segment_even=1000, max_batch=1) as c:
        assert c.verify_range(a, b)[1] == oracle.stats_line(a, b, oracle.SIEVE)
