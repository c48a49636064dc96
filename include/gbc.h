/*
 * gbc.h -- C ABI of the GB300 dense Goldbach verify path (and, at the end,
 * the sparse class map cross-check). The measurement probe the bench reports
 * the sieve stages against is a separate library (include/gbc_probe.h).
 *
 * The reference (goldbach-l0) has no FFI: its boundary for this path is the
 * dense run driver's per-segment contract (src/verifier.cpp:1741-2444:
 * prepare_segment_tables / enqueue_sieve / enqueue_large_primes /
 * enqueue_check / collect_slot) under gb::run_gpu (include/verifier.hpp:
 * 71-110). Every entry point below replaces one piece of that contract, as
 * its comment says. Plain C types only; every call returns an int status
 * (GBC_OK = 0, negative = error class) and gbc_last_error() gives the text.
 * Nothing here throws, nothing here falls back to the CPU.
 *
 * Terms: an "even" is an even n to verify; p(n) is the smallest odd prime p
 * with n - p prime (2 for n = 4). A "segment" is a run of consecutive evens
 * [seg_start, seg_end] (inclusive) whose statistics are reported together;
 * a "batch" is up to max_batch segments sieved and checked by one pass of
 * the pipeline; its segments form "runs" (maximal sets of consecutive
 * segments), each with its own HBM-resident mod-30 class map, so one batch
 * can hold many windows of different widths and heights. A "slot" is one of
 * nslots independent sets of device buffers with its own stream, so batch
 * k + 1 can be enqueued while batch k is on the GPU or being collected.
 */
#ifndef GBC_H
#define GBC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBC_OK 0
#define GBC_E_ARG (-1)      /* bad argument (range, size, slot, alignment) */
#define GBC_E_CUDA (-2)     /* a CUDA runtime call failed */
#define GBC_E_DEVICE (-3)   /* a device-side error flag was set */
#define GBC_E_TIMEOUT (-4)  /* a bounded wait ran out */
#define GBC_E_STATE (-5)    /* call out of order (collect without enqueue, ...) */
#define GBC_E_OVERFLOW (-6) /* a fixed-capacity output overflowed */

#define GBC_NCAND 1205      /* odd primes 3..9781 (include/config.hpp:81-86 MAX_GB_PRIME) */
#define GBC_MAX_CAND 9781u
#define GBC_NCLASS 15       /* even classes r = n mod 30 = 0, 2, ..., 28 */
#define GBC_GBINS 1024      /* gap histogram bins g / 2 (include/gstats.hpp:78 GAPS30_HBINS) */
#define GBC_GTAIL 700u      /* gaps >= 700 are listed with their position (gstats.hpp:77) */
#define GBC_TAIL_CAP 256    /* listed tail gaps per segment */
#define GBC_LEFT_CAP 1024   /* evens per segment without a candidate witness */
#define GBC_RIDGE_CAP 256   /* listed ridges (evens with p(n) >= ridge_min) per segment */
#define GBC_TAIL_T 3000u    /* every funnel member is below it (include/check30.hpp:33 CHECK30_TAIL) */
#define GBC_DEFAULT_SEGMENT 467500000ull /* include/config.hpp:163 DEFAULT_SEGMENT_EVEN */
#define GBC_MAX_LIMIT 18446742974197923840ull /* 2^64 - 2^40 (include/primes.hpp:212) */

/* segment flags */
#define GBC_SEG_LAST 1u     /* the run's last segment: counts end at limit - 1 */
#define GBC_SEG_NOHASH 2u   /* skip the class-map hash */
#define GBC_SEG_VERIFY 4u   /* funnel verify + exact tail instead of p(n) of every even */
#define GBC_SAMPLE_NONE 0xFFFFFFFFu  /* gbc_config.sample_every: no segment gets p(n) of every even */

/* Context configuration (the knobs of include/config.hpp and the GB_*
 * environment, as fields). Zero means "default" for every field. */
typedef struct gbc_config {
    uint64_t limit;          /* largest even any batch will reach: sizes the sieving primes */
    uint64_t segment_even;   /* integer span of a full segment (default 467.5M) */
    uint32_t max_batch;      /* segments per batch the slots are sized for (default 8, at most 256) */
    uint32_t tile_log2;      /* log2 of shared-memory tile bits per class (14..20, default 20); see tile_bits */
    uint32_t p_mid;          /* primes <= p_mid: shared-memory tiles; above: large-prime kernel (default 2^22) */
    uint32_t want_pn;        /* 1: slots also hold a per-even u16 p(n) buffer */
    int32_t device;          /* CUDA device ordinal (default 0) */
    uint32_t max_runs;       /* runs per batch the slots are sized for (a run: consecutive segments
                                with one class map; windows that do not touch are separate runs);
                                default max_batch, at most max_batch */
    uint32_t hl_mode;        /* prime-multiplier hit lists: 0 auto (on when a batch spans >= 1e9
                                integers), 1 on, 2 off */
    uint32_t mtab_max_gb;    /* HBM budget of the prime-multiplier table (default 48 GB); primes below
                                limit / (30 * budget) keep the read-before-mark kernel */
    uint32_t nslots;         /* independent slots (default 2, 2..GBC_MAX_SLOTS) */
    uint32_t sample_every;   /* run driver: every sample_every-th segment of a run (segment 0 always)
                                gets p(n) of every even, the others the funnel verify + exact tail
                                (GB_STATS_SAMPLE, include/gstats.hpp:62); 0 or 1: every segment
                                (default); GBC_SAMPLE_NONE: no segment (verification without the
                                p(n) histogram: counts, gaps, ridges, and the largest p(n) where it
                                reaches the exact tail's bound GBC_TAIL_T, else 0, as the reference's
                                run_pmax over tail counts alone, include/gstats.hpp:690-701) */
    uint32_t plan_funnels;   /* funnels per class of the verify plan (default 8, at most 32; below 6
                                the evens a production segment leaves to the exact continuation can
                                overflow its pending list, and the batch fails closed) */
    uint32_t ridge_min;      /* evens with p(n) >= ridge_min are listed (default 3000,
                                include/config.hpp:104 RIDGE_MIN_DEFAULT) */
    uint32_t launch_mode;    /* 0 or 1: a batch is one replay of the slot's CUDA graph of the whole
                                pipeline (captured at the slot's first batch); 2: the same kernels
                                launched one by one; 3: the plain form (the reference's per-segment
                                pipeline, src/verifier.cpp:2487-2517): a batch's hit lists harvested
                                once, then each segment by its own launches of the sieve, large-prime,
                                checker and count kernels (batches of several runs: as 2) */
    uint32_t selfcheck_every;/* every selfcheck_every-th batch that uses hit lists rebuilds its maps
                                without them and compares every word (src/verifier.cpp:2057-2112);
                                a mismatch fails the batch closed. 0: never (default) */
    uint32_t verify_funnels; /* funnels of the plan every word of a chunk takes before the verify
                                kernel gathers the words still without a witness, one per lane, for
                                the plan's other funnels (default 3; at most plan_funnels) */
    uint32_t hl_cap_pct;     /* the hit-list bins' quotas and capacities in percent of their sizing
                                (default 100; lower values make marks take the overflow list, which
                                is cleared after the tiles: for tests of that path) */
    uint32_t test_flags;     /* 0 in production; GBC_TEST_* below, for tests of the failure paths */
    uint32_t tile_bits;      /* bits per shared-memory tile of a class array when set: a multiple of
                                4096 in [2^14, 1835008] (up to 224 KB of shared memory); 0: 2^tile_log2 */
} gbc_config;

/* test_flags: each makes a bounded device wait run out, so a test sees the
 * batch fail closed (gbc_collect: GBC_E_DEVICE) with no fault and the
 * context still usable.
 *   GBC_TEST_STAGING_WAIT  the first wait on every bulk copy into shared
 *                          memory in the tile sieve and the verify checker
 *                          gives up at once; its second wait keeps the
 *                          normal limit, so the copies in flight still land
 *   GBC_TEST_RETRY_LIMIT   the exact checker keeps the first candidate of
 *                          each class only, so evens go to the GPU retry,
 *                          whose search stops after one try */
#define GBC_TEST_STAGING_WAIT 1u
#define GBC_TEST_RETRY_LIMIT 2u

#define GBC_MAX_SLOTS 8

typedef struct gbc_ctx gbc_ctx;

/* Per-segment results (collect_slot + GoldbachStats::add_* inputs,
 * src/verifier.cpp:2402-2444, include/gstats.hpp:507-624). Indices into the
 * candidate list are positions in gbc_candidates(). */
typedef struct gbc_segment_result {
    uint64_t seg_start, seg_end, evens;
    uint64_t cnt_lo, cnt_hi;       /* primes counted: q in [cnt_lo, cnt_hi] (odd) */
    uint64_t twin_hi;              /* twin pairs (q, q + 2) counted for q in [cnt_lo, twin_hi] */
    uint64_t hash_lo, hash_hi;     /* class-map hash range */
    /* p(n) of every even (exact; the smallest witness) */
    uint32_t hist[GBC_NCLASS][GBC_NCAND]; /* evens with p(n) = cand[i], by class r / 2 */
    uint32_t first[GBC_NCAND];     /* (n - seg_start) / 2 of the first such even, or UINT32_MAX */
    uint32_t nleft;                /* evens with no witness <= 9781 (retried on the GPU) */
    uint32_t pad0;
    uint64_t left_n[GBC_LEFT_CAP]; /* those evens ... */
    uint64_t left_p[GBC_LEFT_CAP]; /* ... and their p(n) from the GPU retry (0: none found) */
    /* primes, twins, gaps of q in the count range (count30 + add_gap_segment) */
    uint64_t primes30[8];          /* by residue 1, 7, 11, 13, 17, 19, 23, 29 */
    uint64_t twins[3];             /* lower prime = 11, 17, 29 (mod 30) */
    uint32_t ghist[GBC_GBINS];     /* gaps q - prev(q) by g / 2 */
    uint64_t gmax_key;             /* largest gap: g << 32 | (UINT32_MAX - (lower - hash_lo)) */
    uint32_t ntail;                /* gaps >= 700 listed below (count may exceed the cap: error) */
    uint32_t pad1;
    uint32_t tail_g[GBC_TAIL_CAP];
    uint64_t tail_lo[GBC_TAIL_CAP];/* lower prime of each listed gap */
    uint64_t first_prime, last_prime; /* in the count range (0: none) */
    uint64_t map_hash;             /* sum of splitmix64(q) over primes q in [hash_lo, hash_hi] coprime to 30 */
    uint64_t map_primes;           /* number of those primes */
    /* checker mode of the segment: sampled = 1: hist holds p(n) of every
     * even (check30_xs* + check30_xb, goldbach.cl:2339-3021); sampled = 0:
     * the funnel verify (check30_a) resolved all evens but `pending`, and
     * hist / first hold the exact p(n) of those (check30_b, goldbach.cl:
     * 2210-2306): every even with p(n) >= the plan bound is among them */
    uint32_t sampled;
    uint32_t npend;                /* phase-A pending words (evens with no plan witness) */
    uint64_t pending;              /* phase-A pending evens */
    uint32_t nridge;               /* evens with p(n) >= ridge_min, listed below (RidgeTracker) */
    uint32_t pad3;
    uint32_t ridge_p[GBC_RIDGE_CAP];
    uint64_t ridge_n[GBC_RIDGE_CAP];
    uint32_t err;                  /* device error flags (0 = none) */
    uint32_t pad2;
} gbc_segment_result;

/* Stage times of one batch (device events on the slot's stream). */
typedef struct gbc_batch_times {
    float ms_setup, ms_tile, ms_large, ms_check, ms_count, ms_total;
    float ms_selfcheck;      /* map self-check of this batch (0 when it had none) */
    uint32_t runs;           /* class maps (runs) of the batch */
} gbc_batch_times;

/* Creates a context on cfg->device: the sieving primes up to
 * sqrt(cfg->limit + 3), the pattern and wheel tables, and two slots.
 * Replaces DenseRun's construction (src/verifier.cpp:346-354) and
 * RunSetup::load_base_primes / upload_tables (src/verifier.cpp:633-692,
 * 1361-1440). Returns GBC_OK and *out, or an error: *out is then a
 * context holding the error text for gbc_last_error, which the caller
 * destroys (NULL only when out is NULL or no context could be allocated). */
int gbc_create(const gbc_config *cfg, gbc_ctx **out);

/* Frees every device and host buffer of the context (release_device_objects,
 * src/verifier.cpp). Safe on NULL. */
void gbc_destroy(gbc_ctx *ctx);

/* Text of the last error on this context (ZE_CHECK's message,
 * include/l0_context.hpp:14-20); never NULL. */
const char *gbc_last_error(const gbc_ctx *ctx);

/* The configuration in force, defaults filled in (the values RunSetup
 * resolves in resolve_range / load_base_primes, src/verifier.cpp:573-692). */
int gbc_get_config(const gbc_ctx *ctx, gbc_config *out);

/* The odd candidate primes 3..9781 ascending (gb_primes of
 * RunSetup::load_base_primes, src/verifier.cpp:686-691). Returns the count. */
int gbc_candidates(uint16_t *out, int cap);

/* Enqueues one batch of nseg consecutive segments on a slot: tile sieve,
 * large primes, checker, counts (prepare_segment_tables + enqueue_sieve +
 * enqueue_large_primes + enqueue_check, src/verifier.cpp:1741-2146).
 * seg_bounds holds 2 * nseg evens: [seg_start, seg_end] of each segment,
 * consecutive (seg_start[i+1] = seg_end[i] + 2), all even, 4 <= seg_start,
 * seg_end <= limit <= GBC_MAX_LIMIT. seg_flags (nseg entries or NULL) holds
 * GBC_SEG_* flags; limit is the run's last even (counts stop at limit - 1).
 * Returns at once; the work runs on the slot's stream. */
int gbc_enqueue_batch(gbc_ctx *ctx, int slot, const uint64_t *seg_bounds, const uint32_t *seg_flags, int nseg,
                      uint64_t limit);

/* Enqueues one batch of nseg segments of any windows on a slot, the batched
 * form of gbc_enqueue_batch (the reference enqueues one segment per slot,
 * src/verifier.cpp:1741-2146; here every stage is one persistent launch over
 * all segments and runs of the batch). Segment i is [seg_bounds[2i],
 * seg_bounds[2i+1]] with the same rules as above, and seg_limits[i] is the
 * last even of the window it belongs to (its counts stop at seg_limits[i] -
 * 1 when seg_end = seg_limits[i]). Segments that follow each other
 * (seg_start[i] = seg_end[i-1] + 2) share one class map (a run); any other
 * step starts a new run, so windows may overlap, repeat or come in any
 * order. At most max_runs runs, and their maps must fit the slot's map
 * buffer (max_batch full segments plus a small margin per run);
 * GBC_E_ARG otherwise, with nothing enqueued. */
int gbc_enqueue_segments(gbc_ctx *ctx, int slot, const uint64_t *seg_bounds, const uint32_t *seg_flags,
                         const uint64_t *seg_limits, int nseg);

/* Waits (at most timeout_ms; < 0 waits without a limit) for the slot's
 * batch and copies its nseg results to host memory (collect_slot,
 * src/verifier.cpp:2402-2444). Fails closed with GBC_E_DEVICE on any device
 * error flag and GBC_E_OVERFLOW when a leftover or tail list overflowed.
 * times may be NULL. */
int gbc_collect(gbc_ctx *ctx, int slot, gbc_segment_result *out, int nseg, gbc_batch_times *times,
                int timeout_ms);

/* 1 when the slot's enqueued batch has finished on the GPU (gbc_collect
 * will not wait), 0 while it runs or when the slot holds no batch, or a
 * negative error (the reference polls its check event the same way,
 * src/verifier.cpp:1847-1858). */
int gbc_poll(gbc_ctx *ctx, int slot);

/* Builds the prime-multiplier table for every batch whose evens lie in
 * [lo, hi] now, so no later batch in that range rebuilds it (the reference
 * builds its mtab once at start-up, src/verifier.cpp:1444-1508). Waits for
 * every slot first. A no-op when hit lists are off or the table already
 * covers the range. */
int gbc_prepare(gbc_ctx *ctx, uint64_t lo, uint64_t hi);

/* Counters of the context: launches of its kernels, batches, graph
 * replays, map self-checks, prime-multiplier table builds and their time,
 * and the device bytes the context holds. */
typedef struct gbc_ctx_stats {
    uint64_t launches, batches, graph_replays, selfchecks;
    uint64_t mtab_builds, mtab_bytes;
    double mtab_build_ms;
    uint64_t device_bytes;
    uint64_t p_hl;            /* first hit-listed prime (0: hit lists off) */
    uint32_t sm_count;        /* multiprocessors of the context's device */
    uint32_t hl_overflow;     /* hit-list marks that took the overflow list (counted when hl_cap_pct < 100) */
} gbc_ctx_stats;
int gbc_get_stats(const gbc_ctx *ctx, gbc_ctx_stats *out);

/* Copies segment i's per-even p(n) of the last collected batch of the slot
 * (u16, index (n - seg_start) / 2; 2 for n = 4; 0 only for a counterexample)
 * into host memory. Needs want_pn. evens = the segment's even count. */
int gbc_copy_pn(gbc_ctx *ctx, int slot, int seg, uint16_t *out, uint64_t evens);

/* Device pointer of the slot's per-even p(n) buffer of segment i (or NULL
 * without want_pn), for callers that keep results on the device. */
const uint16_t *gbc_pn_device_ptr(gbc_ctx *ctx, int slot, int seg);

/* The class map of the first run of the slot's last collected batch, for
 * bit-exact validation against an independent primality test (the
 * reference's debug_map validator, docs/PROJECT-REFERENCE.md:615-620):
 * *base (q of class-array bit 0 minus its residue, a multiple of 30), *nblk
 * (bits per class array in use) and *wpc (words per class array); when out
 * is not NULL, 8 * wpc words are copied to it (class k at out + k * wpc,
 * bit t of class k <-> q = base + 30 t + u_k, u = 1, 7, 11, 13, 17, 19, 23,
 * 29). */
int gbc_map_info(gbc_ctx *ctx, int slot, uint64_t *base, uint32_t *nblk, uint32_t *wpc, uint32_t *out,
                 uint64_t out_words);

/* The same for run `run` of the batch (runs numbered in segment order);
 * GBC_E_ARG past the batch's last run. */
int gbc_map_run(gbc_ctx *ctx, int slot, int run, uint64_t *base, uint32_t *nblk, uint32_t *wpc, uint32_t *out,
                uint64_t out_words);

/* The CUDA stream of a slot (a cudaStream_t), for callers that time or
 * order their own work against it. */
void *gbc_stream(gbc_ctx *ctx, int slot);

/* Number of CUDA kernels this context has launched so far. */
uint64_t gbc_launch_count(const gbc_ctx *ctx);

/* Run-level result (RunStats of include/verifier.hpp:30-69, the counts only). */
typedef struct gbc_run_result {
    uint64_t start, limit, evens, segments, batches;
    uint64_t leftovers;          /* evens retried on the GPU beyond 9781 */
    uint64_t pmax;               /* largest p(n) */
    uint64_t primes, twins;      /* in [start + 1, limit - 1] */
    double gpu_seconds;          /* device time of the batch loop */
    double wall_seconds;
} gbc_run_result;

/* Verifies every even in [start, limit] through the per-segment contract
 * above and writes the reference's stats_ref line (tests/stats_ref.cpp:
 * 97-189) into line (NUL-terminated; line may be NULL). pn (host, or NULL)
 * receives p(n) of every even, (limit - start) / 2 + 1 entries; it needs
 * want_pn. The run driver of gb::run_gpu (src/verifier.cpp:2487-2569) as one
 * call: segments of cfg->segment_even, batches of cfg->max_batch, two slots
 * in flight, fail closed on any error. */
int gbc_verify_range(gbc_ctx *ctx, uint64_t start, uint64_t limit, gbc_run_result *res, char *line,
                     uint64_t line_cap, uint16_t *pn);

/* ---- batched windows and the serving loop ---------------------------------
 * Both pack the segments of many windows into shared batches (continuous
 * batching over the context's slots): a window's segments go out in order,
 * windows in arrival order, up to max_batch segments in up to max_runs runs
 * per batch, up to nslots batches on the GPU at once. Each window's
 * statistics are exactly those of a run of that window alone. */

/* Totals of one gbc_verify_windows call. */
typedef struct gbc_windows_summary {
    uint64_t batches, segments, runs;
    double gpu_seconds, wall_seconds;
} gbc_windows_summary;

/* Verifies nwin windows [bounds[2i], bounds[2i+1]] (each with the rules of
 * gbc_verify_range, limit <= the context's limit) in shared batches. res
 * (nwin entries or NULL) gets each window's counts (wall_seconds: from the
 * call to the window's completion); lines (nwin * line_stride bytes or
 * NULL) gets each window's line as gbc_verify_range writes it, window i at
 * lines + i * line_stride; sum (or NULL) the call's totals. The reference
 * has no such call: it runs windows one after another (run_gpu,
 * src/verifier.cpp:2487-2569). */
int gbc_verify_windows(gbc_ctx *ctx, const uint64_t *bounds, int nwin, gbc_run_result *res, char *lines,
                       uint64_t line_stride, gbc_windows_summary *sum);

/* A serving loop over one context: a worker thread owns the context (no
 * other call may use it until gbc_server_stop), admits submitted windows
 * in arrival order into batches as slots free up, and keeps the sieving
 * primes and the prime-multiplier table resident. No counterpart in the
 * reference (its service mode runs one range at a time). */
typedef struct gbc_server gbc_server;

typedef struct gbc_server_stats {
    uint64_t submitted, completed, batches, segments, runs;
    uint32_t max_in_flight;        /* most batches on the GPU at once */
    uint32_t pad;
    double gpu_seconds, wall_seconds;
    uint64_t device_bytes;         /* device memory the context holds */
    uint64_t hbm_budget;
} gbc_server_stats;

/* Starts the loop. The context's whole device footprint (slots, tables,
 * and the prime-multiplier table built now for every window in [lo, hi];
 * hi = 0: none) must fit hbm_budget bytes (0: no budget), else GBC_E_ARG.
 * *out receives the server. */
int gbc_server_start(gbc_ctx *ctx, uint64_t hbm_budget, uint64_t lo, uint64_t hi, gbc_server **out);

/* Queues the window [start, limit] (rules of gbc_verify_range); *id
 * receives its ticket. Any thread. */
int gbc_server_submit(gbc_server *srv, uint64_t start, uint64_t limit, uint64_t *id);

/* Waits at most timeout_ms (< 0: no limit) for window id, then writes its
 * counts, its line (as gbc_verify_range) and the time from its submission
 * to its completion; a ticket can be waited for once. Fails with the
 * worker's error if the loop stopped on one (fail closed). */
int gbc_server_wait(gbc_server *srv, uint64_t id, int timeout_ms, gbc_run_result *res, char *line,
                    uint64_t line_cap, double *latency_ms);

int gbc_server_get_stats(gbc_server *srv, gbc_server_stats *out);

/* The worker's error text (empty when none). */
const char *gbc_server_error(gbc_server *srv);

/* Drains every queued window, stops the worker and frees the server; the
 * context is the caller's again. Returns the worker's error, if any. */
int gbc_server_stop(gbc_server *srv);

/* ---- journaled slices -------------------------------------------------------
 * The reference's slice runner (tools/run_range.sh, docs/PIPELINE.md:12-24,
 * 114-122) on one resident context: [start, limit] in slices of `slice`
 * integers, one journal row per slice: "PASS a b <UTC time> <the --csv
 * key=value line> release=<release>" (" attempts=2" when it passed on the
 * retry), "RETRY a b <time> reason=<code>" for a failed first attempt; a
 * slice that fails twice stops the run with its error. A run resumes after
 * the last slice of the journal's contiguous PASS chain from start. A stop
 * file present before a slice ends the run cleanly (*stopped = 1), the
 * resume point intact. */
int gbc_journal_resume(const char *path, uint64_t start, uint64_t *next);
int gbc_run_slices(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t slice, const char *journal,
                   const char *release, const char *stop_file, uint64_t *slices_done, int *stopped);

/* ---- ridge store, records, live snapshot ------------------------------------
 * Host outputs of gbc_verify_range and gbc_run_slices on ctx (the
 * reference's RidgeTracker store, include/ridge.hpp:31-35, 196-237, and its
 * records file, hook and live snapshot, include/gstats.hpp:774-868; the
 * reference opens them from GB_RIDGE_FILE, GB_RECORDS_FILE, GB_STATS_LIVE,
 * GB_RECORD_HOOK, which the command-line front end reads):
 *   ridge_csv  the top 30 ridges, "rank,even,p,q,segment_start,found_unix"
 *              rows, loaded now (every row re-proved on the CPU: p, n - p
 *              prime, no smaller witness), rewritten atomically at the end
 *              of a run whose ridges changed it
 *   records    appended with one line per RECORD (p(n) > 9781), BEYOND or
 *              SP (the campaign's first even with p(n) = p for a p whose
 *              first occurrence is unknown below 4e18; an SP line already in
 *              the file marks p as found) event, each re-proved by a CPU scan
 *   live_json  a one-line JSON snapshot, at most every 2 s and at the end
 *   hook       run in the background per event as `hook KIND P N Q CHECK`
 * NULL or "" turns one off; all NULL detaches the outputs. */
int gbc_set_outputs(gbc_ctx *ctx, const char *ridge_csv, const char *records, const char *live_json,
                    const char *hook);

/* The ridge store at path with count more (n, p, segment start) candidates
 * merged (each proved first; floor: the smallest p kept); *kept = rows. */
int gbc_ridges_merge(const char *path, const uint64_t *n, const uint64_t *p, const uint64_t *seg, uint32_t count,
                     uint32_t floor, uint32_t *kept);

/* One record event for (n, p) into the records file: first = 0: RECORD or
 * BEYOND; first = 1: SP when p is one of the unknown-S(p) primes and no SP
 * line for p is in the file. */
int gbc_record_event(const char *records, const char *hook, uint64_t n, uint64_t p, int first);

/* p(n) by an ascending Miller-Rabin scan on the CPU (0: none <= n / 2). */
uint64_t gbc_pn_exact(uint64_t n);

/* ---- campaign statistics ------------------------------------------------------
 * The reference's campaign statistics files (GoldbachStats, include/gstats.hpp:
 * 507-1342), in its formats byte for byte:
 *   state       "statistics state v2": tail_t, covered ranges, evens, primes and
 *               twins by residue, first occurrences, evens beyond 9781, the
 *               sampled p(n) histogram and the tail counts per class n mod 30,
 *               the class-less tail of unsampled segments
 *   state.gaps  "prime gap state v1" (GapStats): gap ranges, counts, sums of
 *               g^1..g^4, the walk histogram, the largest gap, gaps >= 700
 *   log         one GBSTATS v2 line per merged run (gstats.hpp:913-969); a
 *               GBPSAMP row (the run's p(n) sample) for a covered range run
 *               again and a GBGAPS row when that run's gaps were not in the
 *               gap state yet (a backfill)
 * A passed run is merged once (GoldbachStats::commit, gstats.hpp:715-772):
 * under an exclusive lock on state.lock the state is re-read; a run that
 * overlaps a covered range is not merged again; the gap state is written
 * before the main state, each atomically and durably (temporary file, fsync,
 * rename); a damaged, cut-off or incompatible state is refused and left
 * unchanged. Runs that start below 1e6 keep no campaign statistics
 * (STATS_MIN_START, gstats.hpp:139). */

/* Attaches campaign statistics to ctx: every run of gbc_verify_range and of
 * gbc_run_slices that passes and starts at >= 1e6 is merged into state and
 * logged in log, and the run's line is its GBSTATS v2 line as logged.
 * version: the lines' version= field (NULL: this library's); gaps = 0 keeps no
 * gap statistics (the reference's GB_GAPS=0). The files are read now: a
 * damaged or incompatible state is GBC_E_STATE, nothing attached. state =
 * NULL detaches. */
int gbc_set_stats(gbc_ctx *ctx, const char *state, const char *log, const char *version, int gaps);

/* The statistics half of the per-segment contract without a context: the
 * results of one run [start, limit] (nseg segments covering it in order, as
 * gbc_collect returns them; start >= 1e6) merged into state and log as
 * above (collect_stats + finish_run + commit, src/verifier.cpp:1012-1045,
 * 2553-2563). line (may be NULL) gets the run's GBSTATS v2 line, *merged (may
 * be NULL) 1 when the run was merged, 0 when it overlapped a covered range;
 * err (may be NULL) the message of a failure: GBC_E_ARG for results that do
 * not cover the run, GBC_E_STATE for a coverage failure in a segment or a
 * damaged, unreadable or unwritable state (the files are then unchanged). */
int gbc_stats_commit(const char *state, const char *log, const char *version, int gaps, uint64_t start,
                     uint64_t limit, const gbc_segment_result *segs, int nseg, char *line, uint64_t line_cap,
                     int *merged, char *err, size_t err_cap);

/* ---- allocation-free class map ---------------------------------------------
 * This entry point has no counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: code inside another framework's
 * memory pool with a fixed device budget (an allocation outside the pool is
 * refused or breaks the pool's accounting), and latency-critical paths where
 * cudaMalloc's implicit device-wide synchronization is not acceptable. It
 * needs no gbc_ctx.
 *
 * Builds the exact mod-30 class map of q in [q_lo, q_hi] (the tile sieve's
 * output: bit t of class array k <-> q = base + 30 t + u_k, u = 1, 7, 11,
 * 13, 17, 19, 23, 29, class k at d_map + k * wpc) into d_map, a device
 * buffer of map_words u32 the caller owns, on the given CUDA stream (a
 * cudaStream_t; NULL = the default stream). Bits t < *nblk_out are exact;
 * bits t >= *nblk_out (up to 32 * wpc) are zero. d_primes (device,
 * caller-owned) holds every odd prime 3, 5, 7, ... up to max_prime,
 * ascending (nprimes of them; a count that differs from the number of odd
 * primes <= max_prime is rejected), and max_prime^2 >= q_hi. *base_out,
 * *nblk_out and *wpc_out (each may be NULL) receive the layout; the call
 * returns them and GBC_E_ARG without launching anything when map_words <
 * 8 * wpc, so a caller can size d_map first. err (may be NULL) receives a
 * message on any error.
 *
 * Limits: nprimes <= GBC_NOALLOC_MAX_PRIMES (131072 primes: q_hi up to
 * about 3e12) and q_hi - q_lo <= GBC_NOALLOC_MAX_SPAN (2^30); larger
 * requests are rejected with GBC_E_ARG before any CUDA call. The sieve's
 * scratch (a reciprocal and eight first class bits per prime: 4.5 MiB) is a
 * fixed device array inside this library, which every GPU that loads the
 * library keeps until the process exits; the pattern words of the primes
 * 7..67 are a constant device table of the library. Every call looks up
 * the array's device address on the current device (cudaGetSymbolAddress);
 * the first call on a device also loads this library's device code there,
 * so make the first call on each device before any stream capture. Every
 * call uses the same array and keeps nothing from the last call (each word
 * a kernel reads is written earlier in the same call): calls whose kernels
 * overlap on the GPU (two streams, or two threads) race on it and must be
 * ordered by the caller. This function calls no cudaMalloc, cudaFree or
 * other allocating routine. */
#define GBC_NOALLOC_MAX_PRIMES 131072u
#define GBC_NOALLOC_MAX_SPAN 1073741824ull
int gbc_class_map_noalloc(uint64_t q_lo, uint64_t q_hi, const uint32_t *d_primes, uint32_t nprimes,
                          uint32_t max_prime, uint32_t *d_map, uint64_t map_words, uint64_t *base_out,
                          uint32_t *nblk_out, uint32_t *wpc_out, void *stream, char *err, size_t err_cap);

/* ---- sparse class map: an independent verify-only cross-check ---------------
 * The reference's opt-in sparse path (`--sparse`; include/sparse.hpp:1-33
 * geometry, src/sparse.cpp:840-973 run_gpu_sparse, kernels/sparse.cl).
 * Every even n needs one certified prime q = n - p, so the map holds only
 * the q of K = 12 residue classes c_k mod M = 30030 (0.04% of the integers),
 * chosen so that every even class r = n mod M reaches at least one of them
 * (r - c_k a unit mod M); the candidates p <= pmax of those residues then
 * verify an even through a set map bit. It shares no map, sieve or checker
 * with the dense path and keeps no statistics: it verifies. Evens the GPU
 * leaves are resolved by an ascending Miller-Rabin scan on the CPU.
 *
 * Geometry (all integers): segment s verifies n in [N_s, N_s + M dlt),
 * N_s = N_0 + s M dlt, N_0 = start rounded down to a multiple of M; class
 * k's bit t <-> q = N_s - M TB + c_k + M t, t < dl + TB (dl <= dlt: the
 * segment's evens per class); even n = N_s + r + M i; a candidate
 * p = ((r - c_k) mod M) + M a tests bit t = i + TB - a - [r < c_k].
 * Valid for start - M (TB + 1) > sqrt(limit) and start > pmax (the map's q
 * above every sieving prime); lower starts are GBC_E_ARG ("use the dense
 * path"). */
typedef struct gbc_sparse gbc_sparse;   /* one call at a time per context */

typedef struct gbc_sparse_config {
    uint64_t limit;     /* largest even any call verifies (sizes the sieving primes) */
    uint32_t dlt_log2;  /* evens per even class and segment = 2^dlt_log2, 12..26; 0 = 26 (1.0e12 evens) */
    uint32_t pmax;      /* candidate bound, 1e5..2e8; 0 = 40,000,000 (about 413 primes per residue) */
    uint32_t group_cap; /* plan entries the GPU tests per even class (0 = all); fewer leaves evens to the CPU */
    int device;
    uint32_t host_only; /* 1: residues and plan only, no device (geometry and plan queries; the rest GBC_E_STATE) */
    uint32_t reserved[3];
} gbc_sparse_config;

typedef struct gbc_sparse_result {
    uint64_t evens;      /* evens in [start, limit] */
    uint64_t pending;    /* evens the GPU left, each resolved on the CPU (the reference's leftovers) */
    uint64_t map_primes; /* set map bits summed over the segments */
    uint64_t groups;     /* plan entries tested, summed over the checker's warps */
    uint64_t segments;
    double ms_sieve;     /* GPU time: first bits and tiles (primes below 2^20) */
    double ms_large;     /* GPU time: primes from 2^20 */
    double ms_check;     /* GPU time: the checker */
    double ms_total;     /* wall time of the segment loop, CPU resolution included */
} gbc_sparse_result;

/* Builds the residues (checked to reach every even class), the sieving
 * primes up to sqrt(limit), the inverse table mod M and the checker plan:
 * per even class, the candidates grouped by (class k, window word o: the
 * candidates whose offset is 32 o + 0..31), the fullest groups first, each
 * group stored as plan entries of up to six offsets in ascending order;
 * every candidate is decoded back to p and proved prime, <= pmax and in a
 * usable class before the plan is uploaded (the reference's
 * validate_plan_scm). On an error *out holds a context with the error text
 * for gbc_sparse_last_error (destroy it), or NULL when cfg or out is NULL. */
int gbc_sparse_create(const gbc_sparse_config *cfg, gbc_sparse **out);
void gbc_sparse_destroy(gbc_sparse *sp);
const char *gbc_sparse_last_error(const gbc_sparse *sp);

/* M, K, the K residues (res: K entries), TB, dlt and pmax; any may be NULL. */
int gbc_sparse_geometry(const gbc_sparse *sp, uint32_t *M, uint32_t *K, uint32_t *res, uint32_t *tb, uint32_t *dlt,
                        uint32_t *pmax);

/* Verifies every even of [start, limit] (start rounded up, limit down to
 * even): per segment the map (tiles, then large primes), the checker, and
 * the CPU for the evens it left. Fails closed: GBC_E_DEVICE on a device
 * error flag or when the checker's even count differs from the range's,
 * GBC_E_OVERFLOW when a segment leaves more than 2^20 words pending, and
 * GBC_E_STATE for an even with no Goldbach pair (a counterexample). */
int gbc_sparse_verify(gbc_sparse *sp, uint64_t start, uint64_t limit, gbc_sparse_result *res);

/* The evens the last gbc_sparse_verify left to the CPU, ascending: up to
 * cap into out, *count (may be NULL) = all of them. */
int gbc_sparse_pending(const gbc_sparse *sp, uint64_t *out, uint64_t cap, uint64_t *count);

/* The map of the segment at n0 (a multiple of M, n0 - M (TB + 1) above
 * sqrt(limit)) with dl (1..dlt) evens per class: K rows of row_words =
 * (dl + TB + 31) / 32 words, row k at out + k * row_words, bits at and
 * above dl + TB zero. out_words < K * row_words: GBC_E_ARG. */
int gbc_sparse_map(gbc_sparse *sp, uint64_t n0, uint32_t dl, uint32_t *out, uint64_t out_words);

/* For each even n = start + 2 j, j < count (all in one segment's reach:
 * n - (start rounded down to a multiple of M) < M dlt), the first candidate
 * p in plan order (gbc_sparse_plan) whose q = n - p has its map bit set,
 * within the first group_cap entries; 0 = none. */
int gbc_sparse_witness(gbc_sparse *sp, uint64_t start, uint32_t count, uint32_t *p_out);

/* The cross-check in journaled slices (ci/sparse_crosscheck.sh run: the
 * reference's run_range with GB_SPARSE=1 and its own journal): the rows,
 * resume rule, retry and stop file of gbc_run_slices, each row's csv part
 * "version=gb300-1.0 path=sparse limit= start= segments= leftovers=
 * result=PASS ... stats=0". Coverage of both journals from a start is
 * gbc_journal_resume on each (ci/sparse_crosscheck.sh status). */
int gbc_sparse_run_slices(gbc_sparse *sp, uint64_t start, uint64_t limit, uint64_t slice, const char *journal,
                          const char *release, const char *stop_file, uint64_t *slices_done, int *stopped);

/* Even class r's (r even, < M) candidates p in plan order (entries in
 * order, within an entry ascending offset) with their entry index; returns
 * how many there are, writing at most cap. */
int gbc_sparse_plan(const gbc_sparse *sp, uint32_t r, uint32_t *p_out, uint32_t *group_out, int cap);

#ifdef __cplusplus
}
#endif

#endif /* GBC_H */
