"""ctypes binding of the GB300 dense Goldbach verify path (include/gbc.h).

The product path is libgbc.so next to this file; importing this module does
not load it. `load()` loads it and raises if it is missing (there is no CPU
fallback). `Context` wraps one gbc_ctx: the per-segment contract
(enqueue_batch / collect, the reference's enqueue/collect_slot,
src/verifier.cpp:1741-2444) and the whole-range call verify_range
(gb::run_gpu, include/verifier.hpp:71-110).
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbc.so")

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

ERRORS = {0: "ok", -1: "argument", -2: "cuda", -3: "device flag", -4: "timeout", -5: "state", -6: "overflow"}


class Config(C.Structure):
    _fields_ = [("limit", C.c_uint64), ("segment_even", C.c_uint64), ("max_batch", C.c_uint32),
                ("tile_log2", C.c_uint32), ("p_mid", C.c_uint32), ("want_pn", C.c_uint32),
                ("device", C.c_int32), ("large_pass_mb", C.c_uint32), ("hl_mode", C.c_uint32),
                ("mtab_max_gb", C.c_uint32), ("hl_pass_mb", C.c_uint32), ("sample_every", C.c_uint32),
                ("plan_funnels", C.c_uint32), ("ridge_min", C.c_uint32)]


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
                ("ms_check", C.c_float), ("ms_count", C.c_float), ("ms_total", C.c_float)]


class RunResult(C.Structure):
    _fields_ = [("start", C.c_uint64), ("limit", C.c_uint64), ("evens", C.c_uint64), ("segments", C.c_uint64),
                ("batches", C.c_uint64), ("leftovers", C.c_uint64), ("pmax", C.c_uint64),
                ("primes", C.c_uint64), ("twins", C.c_uint64), ("gpu_seconds", C.c_double),
                ("wall_seconds", C.c_double)]


# every entry point of include/gbc.h: name -> (restype, argtypes)
SIGNATURES = {
    "gbc_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "gbc_destroy": (None, [C.c_void_p]),
    "gbc_last_error": (C.c_char_p, [C.c_void_p]),
    "gbc_get_config": (C.c_int, [C.c_void_p, C.POINTER(Config)]),
    "gbc_candidates": (C.c_int, [C.POINTER(C.c_uint16), C.c_int]),
    "gbc_enqueue_batch": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.c_int,
                                    C.c_uint64]),
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
    "gbc_class_map_noalloc": (C.c_int, [C.c_uint64, C.c_uint64, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                        C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32), C.c_void_p, C.c_char_p, C.c_size_t]),
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
    """One gbc_ctx: sieving primes for `limit`, two slots of `max_batch`
    segments of `segment_even` integers."""

    def __init__(self, limit, segment_even=DEFAULT_SEGMENT, max_batch=8, tile_log2=0, p_mid=0, want_pn=False,
                 device=0, large_pass_mb=0, hl_mode=0, mtab_max_gb=0, hl_pass_mb=0, sample_every=0,
                 plan_funnels=0, ridge_min=0):
        self.lib = load()
        cfg = Config(limit=limit, segment_even=segment_even, max_batch=max_batch, tile_log2=tile_log2,
                     p_mid=p_mid, want_pn=1 if want_pn else 0, device=device, large_pass_mb=large_pass_mb,
                     hl_mode=hl_mode, mtab_max_gb=mtab_max_gb, hl_pass_mb=hl_pass_mb,
                     sample_every=sample_every, plan_funnels=plan_funnels, ridge_min=ridge_min)
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

    def collect(self, slot, nseg, timeout_ms=600000):
        out = (SegmentResult * nseg)()
        t = BatchTimes()
        self._check(self.lib.gbc_collect(self.h, slot, out, nseg, C.byref(t), timeout_ms))
        return list(out), t

    def copy_pn(self, slot, seg, evens):
        buf = (C.c_uint16 * evens)()
        self._check(self.lib.gbc_copy_pn(self.h, slot, seg, buf, evens))
        return buf

    def map(self, slot):
        """(base, nblk, wpc, words) of the slot's last collected class map;
        words is a u32 array of 8 * wpc entries."""
        base, nblk, wpc = C.c_uint64(), C.c_uint32(), C.c_uint32()
        self._check(self.lib.gbc_map_info(self.h, slot, C.byref(base), C.byref(nblk), C.byref(wpc), None, 0))
        words = (C.c_uint32 * (8 * wpc.value))()
        self._check(self.lib.gbc_map_info(self.h, slot, None, None, None, words, len(words)))
        return base.value, nblk.value, wpc.value, words

    def stream(self, slot):
        return self.lib.gbc_stream(self.h, slot)

    def launches(self):
        return self.lib.gbc_launch_count(self.h)

    def verify_range(self, start, limit, want_pn=False):
        """Returns (RunResult, stats_ref line, p(n) array or None)."""
        res = RunResult()
        line = C.create_string_buffer(1 << 16)
        pn = None
        if want_pn:
            pn = (C.c_uint16 * ((limit - start) // 2 + 1))()
        self._check(self.lib.gbc_verify_range(self.h, start, limit, C.byref(res), line, len(line), pn))
        return res, line.value.decode(), pn


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
