"""ctypes binding of the GB300 dense Goldbach verify path (include/gbc.h).

The product path is libgbc.so next to this file; importing this module does
not load it. `load()` loads it and raises if it is missing (there is no CPU
fallback). `Context` wraps one gbc_ctx: the per-segment contract
(enqueue_batch / enqueue_segments / collect, the reference's
enqueue/collect_slot, src/verifier.cpp:1741-2444) and the whole-range call
verify_range (gb::run_gpu, include/verifier.hpp:71-110). `Sparse` wraps the
sparse class map cross-check (gbc_sparse_*, the reference's --sparse path).
`smem_atomic_peak` calls the measurement library libgbc_probe.so (not part of
the verify path): the shared-memory atomic roof the bench reports the sieve
stages against.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbc.so")
PROBE_PATH = os.path.join(HERE, "libgbc_probe.so")

NCAND = 1205
NCLASS = 15
GBINS = 1024
TAIL_CAP = 256
LEFT_CAP = 1024
RIDGE_CAP = 256
TAIL_T = 3000
DEFAULT_SEGMENT = 467_500_000
MAX_LIMIT = 18446742974197923840
SEG_NOHASH = 2
SEG_VERIFY = 4
SAMPLE_NONE = 0xFFFFFFFF  # Config.sample_every: no segment gets p(n) of every even (GBC_SAMPLE_NONE)
TEST_STAGING_WAIT = 1
TEST_RETRY_LIMIT = 2
MAX_SLOTS = 8

ERRORS = {0: "ok", -1: "argument", -2: "cuda", -3: "device flag", -4: "timeout", -5: "state", -6: "overflow"}


class Config(C.Structure):
    _fields_ = [("limit", C.c_uint64), ("segment_even", C.c_uint64), ("max_batch", C.c_uint32),
                ("tile_log2", C.c_uint32), ("p_mid", C.c_uint32), ("want_pn", C.c_uint32),
                ("device", C.c_int32), ("max_runs", C.c_uint32), ("hl_mode", C.c_uint32),
                ("mtab_max_gb", C.c_uint32), ("nslots", C.c_uint32), ("sample_every", C.c_uint32),
                ("plan_funnels", C.c_uint32), ("ridge_min", C.c_uint32), ("launch_mode", C.c_uint32),
                ("selfcheck_every", C.c_uint32), ("verify_funnels", C.c_uint32), ("hl_cap_pct", C.c_uint32),
                ("test_flags", C.c_uint32), ("tile_bits", C.c_uint32)]


class SegmentResult(C.Structure):
    _fields_ = [("seg_start", C.c_uint64), ("seg_end", C.c_uint64), ("evens", C.c_uint64),
                ("cnt_lo", C.c_uint64), ("cnt_hi", C.c_uint64), ("twin_hi", C.c_uint64),
                ("hash_lo", C.c_uint64), ("hash_hi", C.c_uint64),
                ("hist", (C.c_uint32 * NCAND) * NCLASS), ("first", C.c_uint32 * NCAND),
                ("nleft", C.c_uint32), ("pad0", C.c_uint32),
                ("left_n", C.c_uint64 * LEFT_CAP), ("left_p", C.c_uint64 * LEFT_CAP),
                ("primes30", C.c_uint64 * 8), ("twins", C.c_uint64 * 3), ("ghist", C.c_uint32 * GBINS),
                ("gmax_key", C.c_uint64), ("ntail", C.c_uint32), ("pad1", C.c_uint32),
                ("tail_g", C.c_uint32 * TAIL_CAP), ("tail_lo", C.c_uint64 * TAIL_CAP),
                ("first_prime", C.c_uint64), ("last_prime", C.c_uint64),
                ("map_hash", C.c_uint64), ("map_primes", C.c_uint64),
                ("sampled", C.c_uint32), ("npend", C.c_uint32), ("pending", C.c_uint64),
                ("nridge", C.c_uint32), ("pad3", C.c_uint32), ("ridge_p", C.c_uint32 * RIDGE_CAP),
                ("ridge_n", C.c_uint64 * RIDGE_CAP), ("err", C.c_uint32), ("pad2", C.c_uint32)]


class BatchTimes(C.Structure):
    _fields_ = [("ms_setup", C.c_float), ("ms_tile", C.c_float), ("ms_large", C.c_float),
                ("ms_check", C.c_float), ("ms_count", C.c_float), ("ms_total", C.c_float),
                ("ms_selfcheck", C.c_float), ("runs", C.c_uint32)]


class CtxStats(C.Structure):
    _fields_ = [("launches", C.c_uint64), ("batches", C.c_uint64), ("graph_replays", C.c_uint64),
                ("selfchecks", C.c_uint64), ("mtab_builds", C.c_uint64), ("mtab_bytes", C.c_uint64),
                ("mtab_build_ms", C.c_double), ("device_bytes", C.c_uint64), ("p_hl", C.c_uint64),
                ("sm_count", C.c_uint32), ("hl_overflow", C.c_uint32)]


class RunResult(C.Structure):
    _fields_ = [("start", C.c_uint64), ("limit", C.c_uint64), ("evens", C.c_uint64), ("segments", C.c_uint64),
                ("batches", C.c_uint64), ("leftovers", C.c_uint64), ("pmax", C.c_uint64),
                ("primes", C.c_uint64), ("twins", C.c_uint64), ("gpu_seconds", C.c_double),
                ("wall_seconds", C.c_double)]


class WindowsSummary(C.Structure):
    _fields_ = [("batches", C.c_uint64), ("segments", C.c_uint64), ("runs", C.c_uint64),
                ("gpu_seconds", C.c_double), ("wall_seconds", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("batches", C.c_uint64),
                ("segments", C.c_uint64), ("runs", C.c_uint64), ("max_in_flight", C.c_uint32),
                ("pad", C.c_uint32), ("gpu_seconds", C.c_double), ("wall_seconds", C.c_double),
                ("device_bytes", C.c_uint64), ("hbm_budget", C.c_uint64)]


class SparseConfig(C.Structure):
    _fields_ = [("limit", C.c_uint64), ("dlt_log2", C.c_uint32), ("pmax", C.c_uint32), ("group_cap", C.c_uint32),
                ("device", C.c_int32), ("host_only", C.c_uint32), ("reserved", C.c_uint32 * 3)]


class SparseResult(C.Structure):
    _fields_ = [("evens", C.c_uint64), ("pending", C.c_uint64), ("map_primes", C.c_uint64), ("groups", C.c_uint64),
                ("segments", C.c_uint64), ("ms_sieve", C.c_double), ("ms_large", C.c_double),
                ("ms_check", C.c_double), ("ms_total", C.c_double)]


# every entry point of include/gbc.h: name -> (restype, argtypes)
SIGNATURES = {
    "gbc_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "gbc_destroy": (None, [C.c_void_p]),
    "gbc_last_error": (C.c_char_p, [C.c_void_p]),
    "gbc_get_config": (C.c_int, [C.c_void_p, C.POINTER(Config)]),
    "gbc_candidates": (C.c_int, [C.POINTER(C.c_uint16), C.c_int]),
    "gbc_enqueue_batch": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.c_int,
                                    C.c_uint64]),
    "gbc_enqueue_segments": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_uint64), C.c_int]),
    "gbc_poll": (C.c_int, [C.c_void_p, C.c_int]),
    "gbc_prepare": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64]),
    "gbc_get_stats": (C.c_int, [C.c_void_p, C.POINTER(CtxStats)]),
    "gbc_map_run": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                              C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint64]),
    "gbc_collect": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(SegmentResult), C.c_int, C.POINTER(BatchTimes),
                              C.c_int]),
    "gbc_copy_pn": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_uint16), C.c_uint64]),
    "gbc_pn_device_ptr": (C.c_void_p, [C.c_void_p, C.c_int, C.c_int]),
    "gbc_map_info": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                               C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint64]),
    "gbc_stream": (C.c_void_p, [C.c_void_p, C.c_int]),
    "gbc_launch_count": (C.c_uint64, [C.c_void_p]),
    "gbc_verify_range": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.POINTER(RunResult), C.c_char_p,
                                   C.c_uint64, C.POINTER(C.c_uint16)]),
    "gbc_verify_windows": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_int, C.POINTER(RunResult),
                                     C.c_char_p, C.c_uint64, C.POINTER(WindowsSummary)]),
    "gbc_server_start": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(C.c_void_p)]),
    "gbc_server_submit": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]),
    "gbc_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int, C.POINTER(RunResult), C.c_char_p, C.c_uint64,
                                  C.POINTER(C.c_double)]),
    "gbc_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "gbc_server_error": (C.c_char_p, [C.c_void_p]),
    "gbc_server_stop": (C.c_int, [C.c_void_p]),
    "gbc_journal_resume": (C.c_int, [C.c_char_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "gbc_run_slices": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_char_p, C.c_char_p,
                                 C.c_char_p, C.POINTER(C.c_uint64), C.POINTER(C.c_int)]),
    "gbc_set_outputs": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p]),
    "gbc_ridges_merge": (C.c_int, [C.c_char_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)]),
    "gbc_record_event": (C.c_int, [C.c_char_p, C.c_char_p, C.c_uint64, C.c_uint64, C.c_int]),
    "gbc_pn_exact": (C.c_uint64, [C.c_uint64]),
    "gbc_set_stats": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]),
    "gbc_stats_commit": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_uint64, C.c_uint64,
                                   C.c_void_p, C.c_int, C.c_char_p, C.c_uint64, C.POINTER(C.c_int), C.c_char_p,
                                   C.c_size_t]),
    "gbc_class_map_noalloc": (C.c_int, [C.c_uint64, C.c_uint64, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                        C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32), C.c_void_p, C.c_char_p, C.c_size_t]),
    "gbc_sparse_create": (C.c_int, [C.POINTER(SparseConfig), C.POINTER(C.c_void_p)]),
    "gbc_sparse_destroy": (None, [C.c_void_p]),
    "gbc_sparse_last_error": (C.c_char_p, [C.c_void_p]),
    "gbc_sparse_geometry": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)]),
    "gbc_sparse_verify": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.POINTER(SparseResult)]),
    "gbc_sparse_pending": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_uint64, C.POINTER(C.c_uint64)]),
    "gbc_sparse_map": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(C.c_uint32), C.c_uint64]),
    "gbc_sparse_witness": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(C.c_uint32)]),
    "gbc_sparse_plan": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_int]),
    "gbc_sparse_run_slices": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_char_p, C.c_char_p,
                                        C.c_char_p, C.POINTER(C.c_uint64), C.POINTER(C.c_int)]),
}

_lib = None


class GbcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def load(path=LIB_PATH):
    """Loads libgbc.so (once) and declares every entry point. Raises OSError
    when the library is missing: the product has no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def candidates():
    lib = load()
    buf = (C.c_uint16 * NCAND)()
    n = lib.gbc_candidates(buf, NCAND)
    return list(buf[:n])


class Context:
    """One gbc_ctx: sieving primes for `limit`, `nslots` slots of `max_batch`
    segments of `segment_even` integers in at most `max_runs` runs."""

    def __init__(self, limit, segment_even=DEFAULT_SEGMENT, max_batch=8, tile_log2=0, p_mid=0, want_pn=False,
                 device=0, max_runs=0, hl_mode=0, mtab_max_gb=0, nslots=0, sample_every=0,
                 plan_funnels=0, ridge_min=0, launch_mode=0, selfcheck_every=0, verify_funnels=0, hl_cap_pct=0,
                 test_flags=0, tile_bits=0):
        self.lib = load()
        cfg = Config(limit=limit, segment_even=segment_even, max_batch=max_batch, tile_log2=tile_log2,
                     p_mid=p_mid, want_pn=1 if want_pn else 0, device=device, max_runs=max_runs,
                     hl_mode=hl_mode, mtab_max_gb=mtab_max_gb, nslots=nslots,
                     sample_every=sample_every, plan_funnels=plan_funnels, ridge_min=ridge_min,
                     launch_mode=launch_mode, selfcheck_every=selfcheck_every, verify_funnels=verify_funnels,
                     hl_cap_pct=hl_cap_pct, test_flags=test_flags, tile_bits=tile_bits)
        h = C.c_void_p()
        rc = self.lib.gbc_create(C.byref(cfg), C.byref(h))
        self.h = h
        if rc:
            msg = self.lib.gbc_last_error(h).decode() if h else "no context"
            self.close()
            raise GbcError(rc, msg)
        self.cfg = Config()
        self.lib.gbc_get_config(self.h, C.byref(self.cfg))

    def _check(self, rc):
        if rc:
            raise GbcError(rc, self.lib.gbc_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.gbc_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def enqueue_batch(self, slot, segments, limit, flags=None):
        n = len(segments)
        b = (C.c_uint64 * (2 * n))(*[x for s in segments for x in s])
        f = (C.c_uint32 * n)(*flags) if flags else None
        self._check(self.lib.gbc_enqueue_batch(self.h, slot, b, f, n, limit))

    def enqueue_segments(self, slot, segments, limits, flags=None):
        """segments: [(seg_start, seg_end)] of any windows; limits: the last
        even of each segment's window."""
        n = len(segments)
        b = (C.c_uint64 * (2 * n))(*[x for s in segments for x in s])
        lim = (C.c_uint64 * n)(*limits)
        f = (C.c_uint32 * n)(*flags) if flags else None
        self._check(self.lib.gbc_enqueue_segments(self.h, slot, b, f, lim, n))

    def poll(self, slot):
        rc = self.lib.gbc_poll(self.h, slot)
        if rc < 0:
            self._check(rc)
        return rc == 1

    def prepare(self, lo, hi):
        self._check(self.lib.gbc_prepare(self.h, lo, hi))

    def stats(self):
        st = CtxStats()
        self._check(self.lib.gbc_get_stats(self.h, C.byref(st)))
        return st

    def collect(self, slot, nseg, timeout_ms=600000):
        out = (SegmentResult * nseg)()
        t = BatchTimes()
        self._check(self.lib.gbc_collect(self.h, slot, out, nseg, C.byref(t), timeout_ms))
        return list(out), t

    def copy_pn(self, slot, seg, evens):
        buf = (C.c_uint16 * evens)()
        self._check(self.lib.gbc_copy_pn(self.h, slot, seg, buf, evens))
        return buf

    def map(self, slot, run=0):
        """(base, nblk, wpc, words) of a run's class map in the slot's last
        collected batch; words is a u32 array of 8 * wpc entries."""
        base, nblk, wpc = C.c_uint64(), C.c_uint32(), C.c_uint32()
        self._check(self.lib.gbc_map_run(self.h, slot, run, C.byref(base), C.byref(nblk), C.byref(wpc), None, 0))
        words = (C.c_uint32 * (8 * wpc.value))()
        self._check(self.lib.gbc_map_run(self.h, slot, run, None, None, None, words, len(words)))
        return base.value, nblk.value, wpc.value, words

    def stream(self, slot):
        return self.lib.gbc_stream(self.h, slot)

    def launches(self):
        return self.lib.gbc_launch_count(self.h)

    def verify_windows(self, windows, line_cap=1 << 16):
        """[(RunResult, line)] of every window [(start, limit)], packed into
        shared batches; also returns the WindowsSummary."""
        n = len(windows)
        b = (C.c_uint64 * (2 * n))(*[x for w in windows for x in w])
        res = (RunResult * n)()
        lines = C.create_string_buffer(n * line_cap)
        summ = WindowsSummary()
        self._check(self.lib.gbc_verify_windows(self.h, b, n, res, lines, line_cap, C.byref(summ)))
        raw = lines.raw
        out = []
        for i in range(n):
            chunk = raw[i * line_cap:(i + 1) * line_cap]
            out.append((res[i], chunk[:chunk.index(b"\0")].decode()))
        return out, summ

    def run_slices(self, start, limit, slice_, journal, release="gb300-1.0", stop_file=None):
        """Journaled slices (tools/run_range.sh's contract): (slices done now, stopped)."""
        done, stopped = C.c_uint64(), C.c_int()
        self._check(self.lib.gbc_run_slices(self.h, start, limit, slice_, str(journal).encode(), release.encode(),
                                            str(stop_file).encode() if stop_file else None, C.byref(done),
                                            C.byref(stopped)))
        return done.value, bool(stopped.value)

    def set_outputs(self, ridge_csv=None, records=None, live_json=None, hook=None):
        """Ridge store, records file (+ hook) and live snapshot of this
        context's runs; None turns one off."""
        enc = lambda x: str(x).encode() if x else None  # noqa: E731
        self._check(self.lib.gbc_set_outputs(self.h, enc(ridge_csv), enc(records), enc(live_json), enc(hook)))

    def verify_range(self, start, limit, want_pn=False):
        """Returns (RunResult, stats_ref line, p(n) array or None)."""
        res = RunResult()
        line = C.create_string_buffer(1 << 16)
        pn = None
        if want_pn:
            pn = (C.c_uint16 * ((limit - start) // 2 + 1))()
        self._check(self.lib.gbc_verify_range(self.h, start, limit, C.byref(res), line, len(line), pn))
        return res, line.value.decode(), pn


def journal_resume(path, start):
    """Where a journaled run of [start, ...] resumes: after the journal's
    contiguous chain of PASS slices from start."""
    n = C.c_uint64()
    rc = load().gbc_journal_resume(str(path).encode(), start, C.byref(n))
    if rc:
        raise GbcError(rc, "journal")
    return n.value


def ridges_merge(path, entries, floor=3):
    """Merges (n, p, segment start) entries into the ridge store at path
    (each proved on the CPU first); returns the rows kept."""
    k = len(entries)
    n = (C.c_uint64 * max(k, 1))(*[e[0] for e in entries])
    p = (C.c_uint64 * max(k, 1))(*[e[1] for e in entries])
    sg = (C.c_uint64 * max(k, 1))(*[e[2] for e in entries])
    kept = C.c_uint32()
    rc = load().gbc_ridges_merge(str(path).encode(), n, p, sg, k, floor, C.byref(kept))
    if rc:
        raise GbcError(rc, "ridge store")
    return kept.value


def record_event(records, n, p, first=False, hook=None):
    """One record event (RECORD / BEYOND, or SP with first=True) into the
    records file."""
    rc = load().gbc_record_event(str(records).encode(), str(hook).encode() if hook else None, n, p, 1 if first else 0)
    if rc:
        raise GbcError(rc, "record")


def pn_exact(n):
    """p(n) by a CPU Miller-Rabin scan (0: none)."""
    return load().gbc_pn_exact(n)


class Server:
    """The serving loop (gbc_server_*) over a Context; the context must not
    be used otherwise until stop()."""

    def __init__(self, ctx, hbm_budget=0, lo=0, hi=0):
        self.ctx, self.lib = ctx, ctx.lib
        h = C.c_void_p()
        ctx._check(self.lib.gbc_server_start(ctx.h, hbm_budget, lo, hi, C.byref(h)))
        self.h = h

    def _check(self, rc):
        if rc:
            raise GbcError(rc, self.lib.gbc_server_error(self.h).decode() if self.h else "no server")

    def submit(self, start, limit):
        i = C.c_uint64()
        self._check(self.lib.gbc_server_submit(self.h, start, limit, C.byref(i)))
        return i.value

    def wait(self, ticket, timeout_ms=600000):
        """(RunResult, line, latency in ms) of a submitted window."""
        res = RunResult()
        line = C.create_string_buffer(1 << 16)
        lat = C.c_double()
        self._check(self.lib.gbc_server_wait(self.h, ticket, timeout_ms, C.byref(res), line, len(line),
                                             C.byref(lat)))
        return res, line.value.decode(), lat.value

    def stats(self):
        st = ServerStats()
        self._check(self.lib.gbc_server_get_stats(self.h, C.byref(st)))
        return st

    def stop(self):
        if self.h:
            rc = self.lib.gbc_server_stop(self.h)
            self.h = None
            self.ctx._check(rc)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.stop()


def segments_of(start, limit, segment_even):
    """The run driver's segment plan (gb::plan_segments): segment_even
    integers each, the lowest (start < 9788) at most 65536, the last ragged."""
    segs, s = [], start
    while s <= limit:
        ln = segment_even if s >= 9788 else min(segment_even, 65536)
        e = limit if limit - s <= ln - 2 else s + ln - 2
        segs.append((s, e))
        if e >= limit:
            break
        s = e + 2
    return segs


class Sparse:
    """One gbc_sparse: the sparse class map cross-check (include/gbc.h; the
    reference's --sparse path, src/sparse.cpp:840-973). `limit` sizes the
    sieving primes; evens per class and segment 2^dlt_log2; candidates up to
    pmax; group_cap limits the plan entries the GPU tests per even class
    (0: all); host_only builds the residues and the plan without a device."""

    def __init__(self, limit, dlt_log2=0, pmax=0, group_cap=0, device=0, host_only=False):
        self.lib = load()
        cfg = SparseConfig(limit=limit, dlt_log2=dlt_log2, pmax=pmax, group_cap=group_cap, device=device,
                           host_only=1 if host_only else 0)
        h = C.c_void_p()
        rc = self.lib.gbc_sparse_create(C.byref(cfg), C.byref(h))
        self.h = h
        if rc:
            msg = self.lib.gbc_sparse_last_error(h).decode() if h else "no context"
            self.close()
            raise GbcError(rc, msg)
        M, K, tb, dlt, pm = (C.c_uint32() for _ in range(5))
        res = (C.c_uint32 * 16)()
        self._check(self.lib.gbc_sparse_geometry(self.h, C.byref(M), C.byref(K), res, C.byref(tb), C.byref(dlt),
                                                 C.byref(pm)))
        self.M, self.K, self.tb, self.dlt, self.pmax = M.value, K.value, tb.value, dlt.value, pm.value
        self.residues = list(res[:self.K])

    def _check(self, rc):
        if rc:
            raise GbcError(rc, self.lib.gbc_sparse_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbc_sparse_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def verify(self, start, limit):
        r = SparseResult()
        self._check(self.lib.gbc_sparse_verify(self.h, start, limit, C.byref(r)))
        return r

    def pending(self):
        n = C.c_uint64()
        self._check(self.lib.gbc_sparse_pending(self.h, None, 0, C.byref(n)))
        buf = (C.c_uint64 * max(1, n.value))()
        self._check(self.lib.gbc_sparse_pending(self.h, buf, n.value, None))
        return list(buf[:n.value])

    def map(self, n0, dl):
        """The K rows of the segment at n0 (a multiple of M), dl evens per
        class: a list of K lists of row words."""
        rows = (dl + self.tb + 31) // 32
        buf = (C.c_uint32 * (self.K * rows))()
        self._check(self.lib.gbc_sparse_map(self.h, n0, dl, buf, self.K * rows))
        return [list(buf[k * rows:(k + 1) * rows]) for k in range(self.K)]

    def witness(self, start, count):
        buf = (C.c_uint32 * count)()
        self._check(self.lib.gbc_sparse_witness(self.h, start, count, buf))
        return list(buf)

    def run_slices(self, start, limit, slice_, journal, release="gb300-1.0", stop_file=None):
        """The cross-check in journaled slices: (slices verified now, stopped)."""
        done, stopped = C.c_uint64(), C.c_int()
        self._check(self.lib.gbc_sparse_run_slices(self.h, start, limit, slice_, str(journal).encode(),
                                                   release.encode(), str(stop_file).encode() if stop_file else None,
                                                   C.byref(done), C.byref(stopped)))
        return done.value, bool(stopped.value)

    def plan(self, r):
        """Even class r's candidates in plan order: [(p, entry index)]."""
        n = self.lib.gbc_sparse_plan(self.h, r, None, None, 0)
        if n < 0:
            self._check(n)
        p = (C.c_uint32 * max(1, n))()
        g = (C.c_uint32 * max(1, n))()
        self.lib.gbc_sparse_plan(self.h, r, p, g, n)
        return list(zip(p[:n], g[:n]))


_probe = None


def load_probe():
    """The measurement library (include/gbc_probe.h); raises if it is missing."""
    global _probe
    if _probe is None:
        if not os.path.exists(PROBE_PATH):
            raise OSError(f"{PROBE_PATH} is missing: build it with `make -C goldbach-l0_gb300`")
        L = C.CDLL(PROBE_PATH)
        L.gbc_smem_atomic_peak.restype = C.c_int
        L.gbc_smem_atomic_peak.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _probe = L
    return _probe


def smem_atomic_peak(device=0):
    """(atomics per second, atomics per SM clock): the device's
    conflict-free shared-memory atomicAnd throughput."""
    lib = load_probe()
    a, b = C.c_double(), C.c_double()
    rc = lib.gbc_smem_atomic_peak(device, C.byref(a), C.byref(b))
    if rc:
        raise GbcError(rc, "shared-memory atomic probe")
    return a.value, b.value
