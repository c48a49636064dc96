// gb_run.hpp -- C++ run driver over the C ABI of include/gbc.h.
//
// gb::run_gpu mirrors the reference's entry point (include/verifier.hpp:
// 71-110): verify every even in [start_even, limit], return the run's
// statistics, throw on any failure (GbcError carries the C ABI status), and
// never report a PASS that did not happen.
#pragma once
#include <cstdint>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gbc.h"

namespace gb {

struct GbcError : std::runtime_error {
    int code;
    GbcError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// Top-30 smallest-witness records (the reference's RidgeTracker,
// include/ridge.hpp:98-237): (even n, p(n)), p descending, n ascending on ties.
struct Ridge {
    uint64_t n = 0, p = 0;
};

// Totals and timings of one run (RunStats, include/verifier.hpp:30-69).
struct RunStats {
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
    uint64_t gap_count() const;
    bool fully_sampled() const { return evens_sampled_ == evens_; }
    std::string stats_ref_line() const;
    std::string gbstats_line(const char *version) const;
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

// Segments of a run: segment_even integers each, the lowest one short
// (it takes the generic checker), the last one ragged.
std::vector<std::pair<uint64_t, uint64_t>> plan_segments(uint64_t start, uint64_t limit, uint64_t segment_even);

// Runs [start, limit] on an existing context. pn: p(n) of every even, or
// nullptr. sample_every: every sample_every-th segment (segment 0 always)
// gets p(n) of every even, the others the funnel verify + exact tail.
RunStats run_range(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t segment_even, uint32_t max_batch,
                   uint16_t *pn, RunAccumulator *acc_out, uint32_t sample_every = 1);

// The reference's --csv key=value line of a run (src/main.cpp:191-215).
std::string csv_line(const RunStats &st, uint64_t segment);

// Journaled slices (gb_journal.cpp): the resume point of a journal, and a
// run of [start, limit] in slices that appends PASS / RETRY rows.
uint64_t journal_resume(const std::string &path, uint64_t start);
uint64_t run_slices(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t slice, const std::string &journal,
                    const std::string &release, const char *stop_file, FILE *log, int *stopped);

// gb::run_gpu: creates a context, runs, destroys it.
RunStats run_gpu(uint64_t limit, uint64_t segment_even, bool verbose, uint64_t start_even = 4,
                 uint32_t max_batch = 8, uint16_t *pn = nullptr, uint32_t sample_every = 1);

}  // namespace gb
