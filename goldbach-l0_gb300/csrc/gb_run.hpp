// gb_run.hpp -- C++ run driver over the C ABI of include/gbc.h.
//
// run_range is the work of the reference's gb::run_gpu (include/verifier.hpp:
// 71-110) on an existing context: verify every even in [start, limit],
// return the run's statistics, throw on any failure (GbcError carries the C
// ABI status), and never report a PASS that did not happen. gb_verifier.cpp
// wraps it in the reference's own signature (include/gb_verifier.hpp).
#pragma once
#include <cstdint>
#include <cstdio>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gbc.h"
#include "gb_stats.hpp"

namespace gb {

struct GbcError : std::runtime_error {
    int code;
    GbcError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// Top-30 smallest-witness records (the reference's RidgeTracker,
// include/ridge.hpp:63-237): (even n, p(n)), p descending, n descending on ties.
struct Ridge {
    uint64_t n = 0, p = 0;
};

// One segment's share of its batch (gb::run_gpu's per_segment records).
struct SegRecord {
    uint64_t start = 0, end = 0, evens = 0;
    uint32_t leftovers = 0;
    double tile_ms = 0, large_ms = 0, check_ms = 0, wall_ms = 0;  // the segment's share by evens
};

// Totals and timings of one run on a context (the counts of the reference's
// RunStats, include/verifier.hpp:30-69; gb_verifier.cpp fills the
// reference's own struct from it).
struct RangeStats {
    uint64_t start = 0, limit = 0, evens = 0, segments = 0, batches = 0;
    uint64_t leftovers = 0;       // evens settled by the GPU retry beyond 9781
    uint64_t pmax = 0;            // largest p(n) of the run (exact: tail + sampled segments)
    uint64_t primes = 0, twins = 0;
    uint64_t evens_sampled = 0;   // evens with a full p(n) record
    uint64_t tail_evens = 0;      // evens with p(n) >= 3000
    uint64_t pending = 0;         // evens the funnel verify left for the exact continuation
    double gpu_seconds = 0, wall_seconds = 0;
    double tile_ms = 0, large_ms = 0, check_ms = 0, count_ms = 0;
    std::string stats_line;       // tests/stats_ref.cpp's line (every segment sampled), else empty
    std::string gbstats_line;     // the GBSTATS v2 log line of the run (include/gstats.hpp:913-969)
    std::vector<Ridge> ridges;    // the run's top 30 ridges
    bool stats_committed = false; // merged into the context's campaign state (gbc_set_stats)
    std::vector<SegRecord> per_segment;  // filled when run_range is asked for it
};

// Run statistics merged from per-segment results (GoldbachStats::add_* and
// GapStats, include/gstats.hpp:397-624).
class RunAccumulator {
public:
    RunAccumulator() = default;
    RunAccumulator(uint64_t start, uint64_t limit, uint32_t tail_t = GBC_TAIL_T);
    void add_segment(const gbc_segment_result &r);
    uint64_t evens() const { return evens_; }
    uint64_t evens_sampled() const { return evens_sampled_; }
    uint64_t leftovers() const { return leftovers_; }
    uint64_t pending() const { return pending_; }
    uint64_t primes() const;
    uint64_t twins() const;
    uint64_t pmax() const;        // largest p(n) seen (tail or sampled)
    uint64_t tail_evens() const;
    uint64_t count_ge(uint64_t p) const;               // evens with p(n) >= p (p >= the tail bound)
    std::pair<uint64_t, uint64_t> pmax_first() const;  // largest p(n) and its first even
    uint64_t gap_count() const;
    bool fully_sampled() const { return evens_sampled_ == evens_; }
    std::string stats_ref_line() const;
    std::string gbstats_line(const char *version) const;
    // the run in the campaign's form (gb_stats.hpp); gaps_on = false leaves
    // the gap statistics out (the reference's GB_GAPS=0)
    RunRecord record(bool gaps_on = true) const;
    const std::vector<Ridge> &ridges() const { return ridges_; }

private:
    void add_gap(uint64_t g, uint64_t upper);
    void note_gap_max(uint64_t g, uint64_t lower);
    void note_tail(uint32_t g, uint64_t c, uint64_t lower);
    void add_beyond(uint64_t n, uint64_t p);
    void note_ridge(uint64_t n, uint64_t p);

    uint64_t start_ = 0, limit_ = 0, evens_ = 0, segments_ = 0, leftovers_ = 0;
    uint32_t tail_t_ = GBC_TAIL_T;
    uint64_t evens_sampled_ = 0, pending_ = 0;
    std::vector<uint16_t> cand_;
    std::vector<uint64_t> samp_;                                  // [15][NCAND], sampled segments
    std::vector<uint64_t> tail_;                                  // [NCAND], p >= tail_t, every segment
    std::vector<uint64_t> tail_cls_;                              // [15][NCAND], p >= tail_t, sampled segments
    std::vector<uint64_t> tail_agg_;                              // [NCAND], p >= tail_t, other segments
    std::vector<std::pair<uint64_t, uint64_t>> beyond_list_;      // (n, p) beyond 9781, in run order
    std::vector<uint64_t> first_all_;                             // first n per candidate, sampled segments
    std::vector<uint64_t> first_tail_;                            // first n per tail candidate, every segment
    std::map<uint64_t, std::pair<uint64_t, uint64_t>> beyond_;    // p -> (count, first n), GPU retry
    uint64_t primes30_[30] = {}, twins30_[30] = {};
    std::vector<uint64_t> ghist_;                                 // even gaps by g / 2
    uint64_t odd_gaps_ = 0;                                       // 3 - 2
    uint64_t gmax_ = 0, gmax_lo_ = 0;
    std::map<uint32_t, std::pair<uint64_t, uint64_t>> tail_gaps_; // g -> (count, first lower)
    std::vector<Ridge> ridges_;
};

// Deterministic 64-bit primality (Miller-Rabin) and p(n) by an ascending
// scan: the CPU re-proof of ridges and record events (gb_records.cpp).
bool is_prime_u64(uint64_t n);
uint64_t pn_exact(uint64_t n);

struct RidgeRow {
    uint64_t n = 0, p = 0, q = 0, seg = 0, found = 0;
};

// The top 30 ridges with every entry proved on the CPU (include/ridge.hpp:
// 63-237): larger p first, the larger even first on ties.
class RidgeStore {
public:
    static constexpr size_t kKeep = 30;
    explicit RidgeStore(uint32_t floor = GBC_TAIL_T) : floor_(floor) {}
    bool consider(uint64_t n, uint64_t p, uint64_t seg, uint64_t found = UINT64_MAX);
    bool load(const std::string &path);
    bool save(const std::string &path);  // rewritten atomically when the top changed
    const std::vector<RidgeRow> &top() const { return top_; }
    uint64_t appends() const { return appends_; }
    uint64_t dropped() const { return dropped_; }

private:
    std::vector<RidgeRow> top_;
    uint32_t floor_;
    uint64_t appends_ = 0, dropped_ = 0;
    bool changed_ = false;
};

class RunAccumulator;

// A context's ridge store, records file (+ hook) and live snapshot.
class Outputs {
public:
    Outputs(const char *ridge_csv, const char *records, const char *live_json, const char *hook,
            uint32_t ridge_floor);
    void add_segment(const gbc_segment_result &r, const std::vector<uint16_t> &cand);
    void note_beyond(uint64_t n, uint64_t p);
    void note_first(uint64_t n, uint64_t p);
    void write_live(uint64_t start, uint64_t limit, uint64_t evens_done, uint64_t evens_total, double elapsed,
                    const RunAccumulator &acc, bool force);
    void finish_run();
    const RidgeStore &ridges() const { return ridges_; }

private:
    void record(uint64_t n, uint64_t p, const char *kind, const char *what);
    std::string ridge_csv_, records_, live_json_, hook_;
    RidgeStore ridges_;
    std::set<uint64_t> sp_seen_;
    std::vector<std::pair<uint64_t, uint64_t>> events_;  // (n, p) recorded by this context
    long long live_t_ = 0;
};

// the outputs attached to a context by gbc_set_outputs, or nullptr
Outputs *outputs_of(gbc_ctx *ctx);

// attaches the reference's ridge store, records file, live snapshot and
// record hook to ctx from its GB_* environment (gb_records.cpp)
void attach_env_outputs(gbc_ctx *ctx);

// the campaign statistics attached to a context by gbc_set_stats, or nullptr;
// stats_gaps_of: whether its runs record their gaps
StatsCampaign *campaign_of(gbc_ctx *ctx);
bool stats_gaps_of(gbc_ctx *ctx);

// the version= field of this library's statistics lines and journal rows
constexpr const char *kVersion = "gb300-1.0";

// runs that start below this keep no campaign statistics (STATS_MIN_START,
// include/gstats.hpp:139)
constexpr uint64_t kStatsMinStart = 1000000;

// Segments of a run: segment_even integers each, the lowest one short
// (it takes the generic checker), the last one ragged.
std::vector<std::pair<uint64_t, uint64_t>> plan_segments(uint64_t start, uint64_t limit, uint64_t segment_even);

// The checker of segment j of a run under gbc_config.sample_every: p(n) of
// every even (0) for every sample_every-th segment from segment 0, the
// funnel verify + exact tail (GBC_SEG_VERIFY) for the others and for every
// segment under GBC_SAMPLE_NONE.
inline uint32_t segment_flag(uint32_t sample_every, size_t j)
{
    if (sample_every == GBC_SAMPLE_NONE) return GBC_SEG_VERIFY;
    return sample_every > 1 && j % sample_every ? GBC_SEG_VERIFY : 0u;
}

// Runs [start, limit] on an existing context. pn: p(n) of every even, or
// nullptr. sample_every: every sample_every-th segment (segment 0 always)
// gets p(n) of every even, the others the funnel verify + exact tail.
RangeStats run_range(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t segment_even, uint32_t max_batch,
                     uint16_t *pn, RunAccumulator *acc_out, uint32_t sample_every = 1, bool per_segment = false);

// The reference's --csv key=value line of a run (src/main.cpp:191-215).
std::string csv_line(const RangeStats &st, uint64_t segment);

// Journaled slices (gb_journal.cpp): the resume point of a journal, and a
// run of [start, limit] in slices that appends PASS / RETRY rows.
uint64_t journal_resume(const std::string &path, uint64_t start);
uint64_t run_slices(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t slice, const std::string &journal,
                    const std::string &release, const char *stop_file, FILE *log, int *stopped);

// The sparse class map cross-check of [start_even, limit] on one gbc_sparse
// context (the work of gb::run_gpu_sparse, src/sparse.cpp:840-973); evens,
// segments, leftovers (evens the GPU left, proved on the CPU) and the stage
// times. No statistics. Throws GbcError.
RangeStats run_sparse(uint64_t limit, bool verbose, uint64_t start_even, uint32_t dlt_log2 = 0);

// The sparse cross-check in journaled slices (ci/sparse_crosscheck.sh run):
// run_slices' rows, resume rule and stop file, each slice through
// gbc_sparse_verify; its csv line carries path=sparse and no statistics.
uint64_t run_sparse_slices(gbc_sparse *sp, uint64_t start, uint64_t limit, uint64_t slice, const std::string &journal,
                           const std::string &release, const char *stop_file, FILE *log, int *stopped);
std::string sparse_csv_line(const RangeStats &st);

}  // namespace gb
