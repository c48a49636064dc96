// gb_run.hpp -- C++ run driver over the C ABI of include/gbc.h.
//
// gb::run_gpu mirrors the reference's entry point (include/verifier.hpp:
// 71-110): verify every even in [start_even, limit], return the run's
// statistics, throw on any failure (GbcError carries the C ABI status), and
// never report a PASS that did not happen.
#pragma once
#include <cstdint>
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

// Totals and timings of one run (RunStats, include/verifier.hpp:30-69).
struct RunStats {
    uint64_t start = 0, limit = 0, evens = 0, segments = 0, batches = 0;
    uint64_t leftovers = 0;   // evens settled by the GPU retry beyond 9781
    uint64_t pmax = 0;        // largest p(n)
    uint64_t primes = 0, twins = 0;
    double gpu_seconds = 0, wall_seconds = 0;
    double tile_ms = 0, large_ms = 0, check_ms = 0, count_ms = 0;
    std::string stats_line;   // tests/stats_ref.cpp's output line for the run
};

// Run statistics merged from per-segment results (GoldbachStats::add_* and
// GapStats, include/gstats.hpp:397-624).
class RunAccumulator {
public:
    RunAccumulator() = default;
    RunAccumulator(uint64_t start, uint64_t limit);
    void add_segment(const gbc_segment_result &r);
    uint64_t evens() const { return evens_; }
    uint64_t leftovers() const { return leftovers_; }
    uint64_t primes() const;
    uint64_t twins() const;
    uint64_t pmax() const;
    uint64_t gap_count() const;
    std::string stats_ref_line() const;

private:
    void add_gap(uint64_t g, uint64_t upper);
    void note_gap_max(uint64_t g, uint64_t lower);
    void note_tail(uint32_t g, uint64_t c, uint64_t lower);
    void add_pn(uint64_t n, uint64_t p);

    uint64_t start_ = 0, limit_ = 0, evens_ = 0, segments_ = 0, leftovers_ = 0;
    std::vector<uint16_t> cand_;
    std::vector<uint64_t> hist_;                                  // [15][NCAND]
    std::vector<uint64_t> first_;                                 // first n per candidate
    std::map<uint64_t, std::pair<uint64_t, uint64_t>> beyond_;    // p -> (count, first n), GPU retry
    uint64_t primes30_[30] = {}, twins30_[30] = {};
    std::vector<uint64_t> ghist_;                                 // even gaps by g / 2
    uint64_t odd_gaps_ = 0;                                       // 3 - 2
    uint64_t gmax_ = 0, gmax_lo_ = 0;
    std::map<uint32_t, std::pair<uint64_t, uint64_t>> tail_;      // g -> (count, first lower)
};

// Segments of a run: segment_even integers each, the lowest one short
// (it takes the generic checker), the last one ragged.
std::vector<std::pair<uint64_t, uint64_t>> plan_segments(uint64_t start, uint64_t limit, uint64_t segment_even);

// Runs [start, limit] on an existing context. pn: p(n) of every even, or nullptr.
RunStats run_range(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t segment_even, uint32_t max_batch,
                   uint16_t *pn, RunAccumulator *acc_out);

// gb::run_gpu: creates a context, runs, destroys it.
RunStats run_gpu(uint64_t limit, uint64_t segment_even, bool verbose, uint64_t start_even = 4,
                 uint32_t max_batch = 8, uint16_t *pn = nullptr);

}  // namespace gb
