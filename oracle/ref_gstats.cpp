// ref_gstats.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product):
// drives the reference's own campaign statistics (GoldbachStats and GapStats
// of the goldbach-l0 header include/gstats.hpp, compiled from the reference
// tree by oracle/Makefile's `ref` target) through a sequence of runs, so the
// tests can compare this repository's statistics files with what the
// reference writes from the same runs.
//
// For each run it feeds GoldbachStats the per-segment inputs its kernels
// would deliver (src/verifier.cpp:1012-1045 collect_stats, 205-237
// resolve_leftovers), computed here on the CPU from the reference's own
// is_prime_u64 (src/primes.cpp):
//   sampled segments   add_full: the p(n) histogram in the statistics plan's
//                      candidate order (make_stats_plan, K = 64);
//   other segments     add_tail: p(n) >= tail_t by p >> 1;
//   every segment      add_first for the wanted tail bins (want_p), the
//                      count30 outputs (count30_limits: primes q in
//                      [s - 3, e - 3], twins with q in [s - 5, e - 5]) and,
//                      with gaps on, add_gap_segment with the walk of the
//                      counted primes (positions from q_first = s - 9781);
//   evens without a candidate witness <= 9781: add_cpu.
// Then finish_run and commit, as DenseRun::assemble_run_stats
// (src/verifier.cpp:2553-2563). Segments follow gb::plan_segments of this
// repository: seg_even integers each, the last one ragged; segment k is
// sampled when k % sample_every == 0 (the reference's rule,
// src/verifier.cpp:2133).
//
// usage: ref_gstats DIR VERSION SAMPLE_EVERY SEG_EVEN  GAPS START LIMIT [GAPS START LIMIT ...]
//   DIR holds goldbach_stats.state (+ .gaps) and goldbach_stats.log; after
//   run i the state and gap state are also copied to DIR/after<i>.state and
//   DIR/after<i>.gaps (when present). Exit 0, or 3 with the reference's
//   exception text when a run throws (a refused, damaged state).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "check30.hpp"
#include "config.hpp"
#include "gstats.hpp"
#include "primes.hpp"

namespace {

void copy_file(const std::string &from, const std::string &to)
{
    std::ifstream in(from, std::ios::binary);
    if (!in) return;
    std::ofstream out(to, std::ios::binary);
    out << in.rdbuf();
}

struct Segment {
    uint64_t s, e;
};

std::vector<Segment> plan_segments(uint64_t start, uint64_t limit, uint64_t seg_even)
{
    std::vector<Segment> v;
    for (uint64_t s = start; s <= limit;) {
        const uint64_t e = limit - s <= seg_even - 2 ? limit : s + seg_even - 2;
        v.push_back({s, e});
        if (e >= limit) break;
        s = e + 2;
    }
    return v;
}

int run_one(const std::string &dir, const char *version, uint32_t sample_every, uint64_t seg_even, bool gaps,
            uint64_t start, uint64_t limit, const std::vector<uint32_t> &gb_all, const gb::StatsPlan &splan,
            uint32_t tail_t)
{
    gb::GoldbachStats st(gb_all, splan, tail_t);
    st.set_run_start(start);
    if (gaps) st.begin_gaps(start);
    const auto segs = plan_segments(start, limit, seg_even);
    // primality of every odd q the run touches: [start - 9781 - 2, limit + 2]
    const uint64_t qlo = (start - gb::MAX_GB_PRIME - 4) | 1, qhi = limit + 3;
    std::vector<uint8_t> isq((qhi - qlo) / 2 + 1);
    for (uint64_t q = qlo; q <= qhi; q += 2) isq[(q - qlo) / 2] = gb::is_prime_u64(q) ? 1 : 0;
    const auto prime = [&](uint64_t q) { return (q & 1) && q >= qlo && q <= qhi && isq[(q - qlo) / 2]; };
    const size_t np = gb_all.size();
    std::vector<uint16_t> pi_of(gb_all.back() / 2 + 1, 0xFFFF);
    for (size_t i = 0; i < np; ++i) pi_of[gb_all[i] / 2] = uint16_t(i);
    // xall position of (class cr, prime index)
    std::vector<int32_t> xpos(15 * np, -1);
    for (uint32_t cr = 0; cr < 15; ++cr) {
        const uint32_t o = splan.xtab[cr], len = splan.xtab[30 + cr];
        for (uint32_t j = 0; j < len; ++j) xpos[cr * np + splan.pidx[o + j]] = int32_t(o + j);
    }
    uint64_t evens = 0, sampled_total = 0;
    for (size_t k = 0; k < segs.size(); ++k) {
        const Segment g = segs[k];
        const uint64_t seg_evens = (g.e - g.s) / 2 + 1;
        const bool sampled = k % sample_every == 0;
        evens += seg_evens;
        if (sampled) sampled_total += seg_evens;
        std::vector<uint32_t> hist(splan.xall.size(), 0), hist_p(gb_all.back() / 2 + 1, 0),
            first_p(gb_all.back() / 2 + 1, ~0u);
        std::vector<std::pair<uint64_t, uint64_t>> cpu;
        const std::vector<uint32_t> &want = st.want_p();
        for (uint64_t n = g.s; n <= g.e; n += 2) {
            uint64_t p = 0;
            for (uint32_t c : gb_all)
                if (prime(n - c)) {
                    p = c;
                    break;
                }
            if (!p) {
                p = gb::pn_exact(n);
                cpu.push_back({n, p});
                continue;
            }
            const uint32_t cr = uint32_t(n % 30) / 2;
            if (sampled) hist.at(size_t(xpos.at(cr * np + pi_of[p / 2]))) += 1;
            else if (p >= tail_t) hist_p[p / 2] += 1;
            const bool wanted = (want[p / 64] >> ((p / 2) & 31)) & 1u;
            if (wanted && first_p[p / 2] == ~0u) first_p[p / 2] = uint32_t((n - g.s) / 2);
        }
        if (sampled) st.add_full(hist.data());
        else st.add_tail(hist_p.data());
        st.add_first(g.s, first_p.data());
        // count30: primes in [s - 3, e - 3], twins (q, q + 2) with q in [s - 5, e - 5]
        const uint64_t q_first = g.s - gb::MAX_GB_PRIME;
        std::vector<uint32_t> cnt(16, 0);
        cnt[11] = ~0u;
        cnt[12] = 0;
        std::vector<uint64_t> ps;
        for (uint64_t q = g.s - 3; q <= g.e - 3; q += 2)
            if (prime(q)) ps.push_back(q);
        static const int res_idx[30] = {-1, 0, -1, -1, -1, -1, -1, 1, -1, -1, -1, 2, -1, 3, -1,
                                        -1, -1, 4, -1, 5, -1, -1, -1, 6, -1, -1, -1, -1, -1, 7};
        for (uint64_t q : ps) cnt[size_t(res_idx[q % 30])] += 1;
        for (uint64_t q = g.s - 5; q <= g.e - 5; q += 2)
            if (prime(q) && prime(q + 2)) cnt[q % 30 == 11 ? 8 : q % 30 == 17 ? 9 : 10] += 1;
        if (!ps.empty()) {
            cnt[11] = uint32_t(ps.front() - q_first);
            cnt[12] = uint32_t(ps.back() - q_first);
        }
        if (gaps) {
            std::vector<uint32_t> gt(2, 0), wh(gb::GAPS30_HBINS, 0);
            uint64_t wmax = 0;
            if (!ps.empty()) wh[0] = 1;
            for (size_t i = 1; i < ps.size(); ++i) {
                const uint64_t gg = ps[i] - ps[i - 1];
                const uint32_t up = uint32_t(ps[i] - q_first);
                wh.at(gg / 2) += 1;
                if (gg >= gb::GAPS30_TAIL) {
                    gt.push_back(up);
                    gt.push_back(uint32_t(gg));
                    gt[0] += 1;
                }
                const uint64_t key = (gg << 32) | uint64_t(uint32_t(~up));
                if (key > wmax) wmax = key;
            }
            st.add_gap_segment(q_first, seg_evens, cnt.data(), gt.data(), &wmax, wh.data());
        }
        st.add_counts(cnt.data());
        for (auto &c : cpu) st.add_cpu(c.first, c.second, sampled);
    }
    st.finish_run(start, limit, evens);
    st.commit(version, sampled_total);
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 8 || (argc - 5) % 3) {
        std::fprintf(stderr, "usage: ref_gstats DIR VERSION SAMPLE_EVERY SEG_EVEN GAPS START LIMIT [...]\n");
        return 2;
    }
    const std::string dir = argv[1];
    const char *version = argv[2];
    const uint32_t sample_every = uint32_t(std::strtoul(argv[3], nullptr, 10));
    const uint64_t seg_even = std::strtoull(argv[4], nullptr, 10);
    setenv("GB_STATS_STATE", (dir + "/goldbach_stats.state").c_str(), 1);
    setenv("GB_STATS_LOG", (dir + "/goldbach_stats.log").c_str(), 1);
    setenv("GB_RECORDS_FILE", (dir + "/goldbach_records.txt").c_str(), 1);
    setenv("GB_STATS_LIVE", (dir + "/goldbach_live.json").c_str(), 1);
    setenv("GB_RECORD_HOOK", "", 1);
    const std::vector<uint32_t> gb_all = gb::odd_primes_up_to(gb::MAX_GB_PRIME);
    const gb::Plan30 plan30 = gb::make_plan30(gb_all, gb::CHECK30_PLAN);
    const uint32_t tail_t = plan30.member_lt;
    const gb::StatsPlan splan = gb::make_stats_plan(gb_all, gb::STATS_K_DEFAULT, tail_t);
    std::printf("tail_t %u\n", tail_t);
    for (int a = 5, run = 1; a + 2 < argc; a += 3, ++run) {
        const bool gaps = std::strtoul(argv[a], nullptr, 10) != 0;
        const uint64_t start = std::strtoull(argv[a + 1], nullptr, 10), limit = std::strtoull(argv[a + 2], nullptr, 10);
        try {
            run_one(dir, version, sample_every, seg_even, gaps, start, limit, gb_all, splan, tail_t);
        } catch (const std::exception &e) {
            std::fprintf(stderr, "run %d: %s\n", run, e.what());
            return 3;
        }
        copy_file(dir + "/goldbach_stats.state", dir + "/after" + std::to_string(run) + ".state");
        copy_file(dir + "/goldbach_stats.state.gaps", dir + "/after" + std::to_string(run) + ".gaps");
    }
    return 0;
}
