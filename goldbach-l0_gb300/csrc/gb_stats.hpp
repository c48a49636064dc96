// gb_stats.hpp -- the campaign statistics of the dense path: a run's exact
// statistics in the reference's campaign form, merged once into a state file
// shared by every run of a campaign.
//
// The files keep the reference's formats byte for byte, so the reference's
// own tools and later reference runs read them (GoldbachStats::commit,
// save_state, load_state, commit_gaps, load_gaps, log_line, gap_fields,
// include/gstats.hpp:715-772, 870-1315):
//   <state>        "goldbach-l0 statistics state v2": tail_t, covered ranges,
//                  evens, primes30, twins30, first occurrences, beyond-list
//                  evens, the sampled p(n) histogram and the tail counts per
//                  class n mod 30, the class-less tail of unsampled segments
//   <state>.gaps   "prime gap state v1": gap ranges, counts, sums of g^k, the
//                  walk histogram, the largest gap, every gap >= 700
//   <log>          one GBSTATS v2 line per merged run; GBPSAMP / GBGAPS rows
//                  for a covered range run again (its p(n) sample; gaps that
//                  were not in the gap state yet)
// A run that overlaps a covered range is not merged again; a damaged or
// incompatible state is refused, never merged into; both files are rewritten
// atomically and durably (temporary file, fsync, rename) under an exclusive
// lock on <state>.lock.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace gb {

using u128 = unsigned __int128;

constexpr uint32_t kGapHistBins = 1024;   // gap histogram bins g / 2
constexpr uint32_t kGapTailMin = 700;     // gaps >= 700 are listed exactly

// Prime gaps of a run or a campaign (GapStats, include/gstats.hpp:397-470).
struct GapTotals {
    uint64_t n = 0;                                          // gaps (one per prime)
    u128 d1 = 0;                                             // sum of g
    std::map<uint32_t, std::pair<uint64_t, uint64_t>> tail;  // g >= 700 -> (count, first lower prime)
    uint64_t gmax = 0, gmax_lo = 0;                          // largest gap, smallest lower prime on ties
    bool all_walked = true;                                  // gmax exact below the tail too
    uint64_t wn = 0;                                         // walked gaps
    u128 wd[4] = {};                                         // walked sums of g, g^2, g^3, g^4
    std::vector<uint64_t> samp = std::vector<uint64_t>(kGapHistBins, 0);  // walked histogram by g / 2

    void note_max(uint64_t g, uint64_t lower);
    void note_tail(uint32_t g, uint64_t count, uint64_t lower);
    bool gmax_exact() const { return gmax >= kGapTailMin || all_walked; }
    void merge(const GapTotals &o);
};

// One run's statistics as the campaign merges them. Histograms are indexed
// by the candidate index (odd primes 3, 5, 7, ... 9781); class cr = n mod 30 / 2.
struct RunRecord {
    uint64_t start = 0, limit = 0, evens = 0, evens_sampled = 0;
    uint32_t tail_t = 3000;
    std::vector<uint64_t> samp;      // [15 * ncand] p(n) of the sampled segments' evens
    std::vector<uint64_t> tail_cls;  // [15 * ncand] p(n) >= tail_t, sampled segments
    std::vector<uint64_t> tail_agg;  // [ncand] p(n) >= tail_t, the other segments (class not kept)
    std::vector<uint64_t> first;     // [ncand] first even of the run with p(n) = p, tail p only (0: none)
    std::vector<std::pair<uint64_t, uint64_t>> beyond;  // (n, p) with p above 9781, in run order
    uint64_t primes30[8] = {}, twins30[3] = {};          // residues 1..29; lower twin 11, 17, 29
    bool gaps_on = true;
    GapTotals gaps;
    uint64_t walk_evens = 0;         // evens of the walked segments

    uint64_t primes() const;
    uint64_t twins() const;
    uint64_t tail_evens() const;
    uint64_t pmax() const;           // largest p(n) >= tail_t of the run (0: none)
};

// The campaign's state file, its gap state and its log.
class StatsCampaign {
public:
    StatsCampaign(std::string state_path, std::string log_path, std::string version, uint32_t tail_t = 3000);

    // Reads both state files as commit would (absent = empty campaign);
    // throws std::runtime_error on a damaged or incompatible one.
    void check() const;

    // Merges a passed run into the campaign, as the reference's commit. When
    // the run overlaps a covered range nothing is merged (the p(n) sample and
    // the gaps of a backfill are logged as GBPSAMP / GBGAPS rows) and *merged
    // is false. Returns the run's GBSTATS v2 line (new_first against the
    // campaign as it was before the merge). Throws std::runtime_error on a
    // damaged state or a failed write (the files are then unchanged).
    std::string commit(const RunRecord &r, bool *merged = nullptr);

    // The run's GBSTATS v2 line against the campaign's current first
    // occurrences (the state is read, not locked or written).
    std::string line(const RunRecord &r) const;

    const std::string &state_path() const { return state_path_; }
    const std::string &log_path() const { return log_path_; }

private:
    std::string state_path_, log_path_, version_;
    uint32_t tail_t_;
};

// GBSTATS v2 line of a run (include/gstats.hpp:913-969), new_first against
// the campaign's first occurrences camp_first ([ncand], 0 = none).
std::string gbstats_line(const RunRecord &r, const std::vector<uint64_t> &camp_first, const std::string &version);

}  // namespace gb
