// gb_run.cpp -- the run driver above the C ABI: gbc_verify_range, the
// campaign statistics calls and gb::run_range of gb_run.hpp.
//
// Follows the reference's DenseRun (src/verifier.cpp:2487-2569): segments
// of segment_even integers, two slots in flight (batch k + 1 is enqueued
// before batch k is collected), per-segment results merged into run
// statistics with the rules of GoldbachStats (include/gstats.hpp:507-772:
// sums, the smallest first occurrence, the largest gap with the smallest
// lower prime on ties, gaps >= 700 with count and first lower prime),
// positive coverage accounting per segment (src/verifier.cpp:2465-2482),
// fail closed on any error. The statistics are printed as the reference's
// run log line (GBSTATS v2, include/gstats.hpp:913-969) and, when every
// segment was sampled, in the format of its CPU oracle tests/stats_ref.cpp:
// 97-189, so a run can be diffed against it line for line.
#include "gb_run.hpp"

#include <algorithm>
#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

void gbh_set_error(gbc_ctx *ctx, const char *msg);                            // gbc_api.cu
void gbh_set_stats(gbc_ctx *ctx, void *p, void (*del)(void *), bool gaps);    // gbc_api.cu
void *gbh_stats(gbc_ctx *ctx, bool *gaps);                                    // gbc_api.cu

namespace gb {

StatsCampaign *campaign_of(gbc_ctx *ctx) { return static_cast<StatsCampaign *>(gbh_stats(ctx, nullptr)); }

bool stats_gaps_of(gbc_ctx *ctx)
{
    bool g = true;
    gbh_stats(ctx, &g);
    return g;
}

namespace {


std::string u128_str(u128 v)
{
    std::string s;
    do {
        s.insert(s.begin(), char('0' + int(v % 10)));
        v /= 10;
    } while (v);
    return s;
}

std::vector<uint16_t> candidates()
{
    std::vector<uint16_t> c(GBC_NCAND);
    gbc_candidates(c.data(), GBC_NCAND);
    return c;
}

// comma-separated counts, an empty entry for 0, trailing zeros cut
// (GoldbachStats::dense_list, include/gstats.hpp:890-903)
std::string dense_list(const std::vector<uint64_t> &v, size_t from = 0)
{
    size_t last = 0;
    for (size_t i = from; i < v.size(); ++i)
        if (v[i]) last = i + 1;
    std::string s;
    for (size_t i = from; i < last; ++i) {
        if (i > from) s += ',';
        if (v[i]) s += std::to_string(v[i]);
    }
    return s;
}

}  // namespace

RunAccumulator::RunAccumulator(uint64_t start, uint64_t limit, uint32_t tail_t)
    : start_(start), limit_(limit), tail_t_(tail_t)
{
    cand_ = candidates();
    samp_.assign(size_t(GBC_NCLASS) * GBC_NCAND, 0);
    tail_.assign(GBC_NCAND, 0);
    tail_cls_.assign(size_t(GBC_NCLASS) * GBC_NCAND, 0);
    tail_agg_.assign(GBC_NCAND, 0);
    first_all_.assign(GBC_NCAND, 0);
    first_tail_.assign(GBC_NCAND, 0);
    ghist_.assign(GBC_GBINS, 0);
    evens_ = (limit - start) / 2 + 1;
    // q = 3 and q = 5 are not in the class map (multiples of 3 and 5): their
    // counts, twins and gaps come from here, exactly, for a run that starts
    // low enough to count them.
    const uint64_t lo = start + 1, hi = limit - 1;
    auto in = [&](uint64_t q) { return q >= lo && q <= hi; };
    if (in(3)) {
        primes30_[3] += 1;
        add_gap(1, 3);
        if (3 + 2 <= limit - 1) twins30_[3] += 1;
    }
    if (in(5)) {
        primes30_[5] += 1;
        add_gap(2, 5);
        if (5 + 2 <= limit - 1) twins30_[5] += 1;
    }
    if (in(7)) add_gap(2, 7);  // 7's predecessor 5 is not in the map
}

void RunAccumulator::add_gap(uint64_t g, uint64_t upper)
{
    if (g / 2 >= GBC_GBINS) throw std::runtime_error("gap above the histogram range");
    if (g & 1) odd_gaps_ += 1;  // 3 - 2: not an entry of the even-gap histogram
    else ghist_[g / 2] += 1;
    note_gap_max(g, upper - g);
    if (g >= GBC_GTAIL) note_tail(uint32_t(g), 1, upper - g);
}

void RunAccumulator::note_gap_max(uint64_t g, uint64_t lower)
{
    if (g > gmax_ || (g == gmax_ && g && lower < gmax_lo_)) {
        gmax_ = g;
        gmax_lo_ = lower;
    }
}

void RunAccumulator::note_tail(uint32_t g, uint64_t c, uint64_t lower)
{
    auto &t = tail_gaps_[g];
    if (!t.first || lower < t.second) t.second = lower;
    t.first += c;
}

void RunAccumulator::add_beyond(uint64_t n, uint64_t p)
{
    auto &b = beyond_[p];
    if (!b.first || n < b.second) b.second = n;
    b.first += 1;
}

void RunAccumulator::note_ridge(uint64_t n, uint64_t p)
{
    const Ridge x{n, p};
    auto better = [](const Ridge &a, const Ridge &b) { return a.p != b.p ? a.p > b.p : a.n > b.n; };
    for (const Ridge &r : ridges_)
        if (r.n == n) return;
    if (ridges_.size() == 30 && !better(x, ridges_.back())) return;
    ridges_.insert(std::upper_bound(ridges_.begin(), ridges_.end(), x, better), x);
    if (ridges_.size() > 30) ridges_.pop_back();
}

void RunAccumulator::add_segment(const gbc_segment_result &r)
{
    // positive accounting: every even of the segment has a p(n) (or, in a
    // verified segment, was resolved by the funnels or has one in the tail)
    uint64_t found = r.nleft;
    for (int cr = 0; cr < GBC_NCLASS; ++cr)
        for (int i = 0; i < GBC_NCAND; ++i) found += r.hist[cr][i];
    const uint64_t want = r.sampled ? r.evens : r.pending;
    if (found != want || r.pending > r.evens)
        throw std::runtime_error("coverage: segment [" + std::to_string(r.seg_start) + ", " +
                                 std::to_string(r.seg_end) + "] accounts for " + std::to_string(found) + " of " +
                                 std::to_string(want) + (r.sampled ? " evens" : " pending evens"));
    for (int cr = 0; cr < GBC_NCLASS; ++cr)
        for (int i = 0; i < GBC_NCAND; ++i) {
            const uint64_t c = r.hist[cr][i];
            if (!c) continue;
            if (r.sampled) samp_[size_t(cr) * GBC_NCAND + i] += c;
            if (cand_[i] >= tail_t_) {
                tail_[i] += c;
                if (r.sampled) tail_cls_[size_t(cr) * GBC_NCAND + i] += c;
                else tail_agg_[i] += c;
            }
        }
    for (int i = 0; i < GBC_NCAND; ++i)
        if (r.first[i] != 0xFFFFFFFFu) {
            const uint64_t n = r.seg_start + 2ull * r.first[i];
            if (r.sampled && (!first_all_[i] || n < first_all_[i])) first_all_[i] = n;
            if (cand_[i] >= tail_t_ && (!first_tail_[i] || n < first_tail_[i])) first_tail_[i] = n;
        }
    if (r.sampled) evens_sampled_ += r.evens;
    else pending_ += r.pending;
    std::vector<std::pair<uint64_t, uint64_t>> left;
    for (uint32_t i = 0; i < r.nleft; ++i) {
        if (!r.left_p[i])
            throw std::runtime_error("no Goldbach partition found for n = " + std::to_string(r.left_n[i]) +
                                     " (reported, never passed)");
        add_beyond(r.left_n[i], r.left_p[i]);
        left.push_back({r.left_n[i], r.left_p[i]});
        ++leftovers_;
    }
    // the campaign keeps them in the order of the evens (the GPU lists them
    // in no fixed order)
    std::sort(left.begin(), left.end());
    for (const auto &e : left)
        if (e.second > GBC_MAX_CAND) beyond_list_.push_back(e);
    for (uint32_t i = 0; i < r.nridge; ++i) note_ridge(r.ridge_n[i], r.ridge_p[i]);
    static const int res[8] = {1, 7, 11, 13, 17, 19, 23, 29};
    for (int k = 0; k < 8; ++k) primes30_[res[k]] += r.primes30[k];
    twins30_[11] += r.twins[0];
    twins30_[17] += r.twins[1];
    twins30_[29] += r.twins[2];
    for (int b = 0; b < GBC_GBINS; ++b) ghist_[b] += r.ghist[b];
    if (r.gmax_key) {
        const uint64_t g = r.gmax_key >> 32;
        const uint64_t lower = r.hash_lo + (0xFFFFFFFFull - (r.gmax_key & 0xFFFFFFFFull));
        note_gap_max(g, lower);
    }
    for (uint32_t i = 0; i < r.ntail; ++i) note_tail(r.tail_g[i], 1, r.tail_lo[i]);
    uint64_t tcount = 0;
    for (int b = GBC_GTAIL / 2; b < GBC_GBINS; ++b) tcount += r.ghist[b];
    if (tcount != r.ntail) throw std::runtime_error("gap tail list does not match the gap histogram");
    segments_ += 1;
}

uint64_t RunAccumulator::primes() const
{
    uint64_t s = 0;
    for (uint64_t v : primes30_) s += v;
    return s;
}

uint64_t RunAccumulator::twins() const
{
    uint64_t s = 0;
    for (uint64_t v : twins30_) s += v;
    return s;
}

uint64_t RunAccumulator::pmax() const
{
    uint64_t m = 0;
    for (int i = 0; i < GBC_NCAND; ++i) {
        uint64_t c = tail_[i];
        for (int cr = 0; cr < GBC_NCLASS; ++cr) c += samp_[size_t(cr) * GBC_NCAND + i];
        if (c) m = cand_[i];
    }
    for (auto &b : beyond_) m = std::max(m, b.first);
    return m;
}

uint64_t RunAccumulator::tail_evens() const
{
    uint64_t t = 0;
    for (uint64_t v : tail_) t += v;
    for (auto &b : beyond_) t += b.second.first;
    return t;
}

uint64_t RunAccumulator::count_ge(uint64_t p) const
{
    uint64_t t = 0;
    for (int i = 0; i < GBC_NCAND; ++i)
        if (cand_[i] >= p) t += tail_[i];
    for (auto &b : beyond_)
        if (b.first >= p) t += b.second.first;
    return t;
}

std::pair<uint64_t, uint64_t> RunAccumulator::pmax_first() const
{
    std::pair<uint64_t, uint64_t> m{0, 0};
    for (int i = GBC_NCAND - 1; i >= 0 && !m.first; --i) {
        if (tail_[i] && first_tail_[i]) m = {cand_[i], first_tail_[i]};
        else if (first_all_[i]) m = {cand_[i], first_all_[i]};
    }
    for (auto &b : beyond_)
        if (b.first > m.first) m = {b.first, b.second.second};
    return m;
}

uint64_t RunAccumulator::gap_count() const
{
    uint64_t n = odd_gaps_;
    for (uint64_t v : ghist_) n += v;
    return n;
}

std::string RunAccumulator::stats_ref_line() const
{
    if (!fully_sampled()) return std::string();
    std::string o;
    char b[128];
    std::snprintf(b, sizeof b, "evens=%" PRIu64 " pmax=%" PRIu64 " primes=%" PRIu64 " twins=%" PRIu64 " primes30=",
                  evens_, pmax(), primes(), twins());
    o += b;
    static const int u[8] = {1, 7, 11, 13, 17, 19, 23, 29};
    for (int i = 0; i < 8; ++i) {
        std::snprintf(b, sizeof b, "%s%" PRIu64, i ? "," : "", primes30_[u[i]]);
        o += b;
    }
    std::snprintf(b, sizeof b, " twins30=%" PRIu64 ",%" PRIu64 ",%" PRIu64, twins30_[11], twins30_[17], twins30_[29]);
    o += b;
    // first occurrences of every p(n) value, ascending p
    std::map<uint64_t, uint64_t> firsts;
    std::vector<uint64_t> tot(GBC_NCAND, 0);
    for (int i = 0; i < GBC_NCAND; ++i) {
        for (int cr = 0; cr < GBC_NCLASS; ++cr) tot[i] += samp_[size_t(cr) * GBC_NCAND + i];
        if (tot[i]) firsts[cand_[i]] = first_all_[i];
    }
    for (auto &bp : beyond_) {
        auto it = firsts.find(bp.first);
        if (it == firsts.end() || bp.second.second < it->second) firsts[bp.first] = bp.second.second;
    }
    o += " first=";
    bool f1 = true;
    for (auto &f : firsts) {
        std::snprintf(b, sizeof b, "%s%" PRIu64 ":%" PRIu64, f1 ? "" : ";", f.first, f.second);
        o += b;
        f1 = false;
    }
    std::vector<uint64_t> hist(tot);
    for (size_t i = 0; i < hist.size(); ++i) {
        auto it = beyond_.find(cand_[i]);
        if (it != beyond_.end()) hist[i] += it->second.first;
    }
    o += " hist=" + dense_list(hist);
    // gaps: count, moments, largest, tail, histogram
    u128 m[4] = {odd_gaps_, odd_gaps_, odd_gaps_, odd_gaps_};  // g = 1
    uint64_t n = odd_gaps_;
    for (size_t i = 0; i < ghist_.size(); ++i) {
        const u128 c = ghist_[i], g = 2 * i, g2 = g * g;
        n += ghist_[i];
        m[0] += c * g;
        m[1] += c * g2;
        m[2] += c * g2 * g;
        m[3] += c * g2 * g2;
    }
    o += " gaps=" + std::to_string(n) + " gmom=" + u128_str(m[0]) + "," + u128_str(m[1]) + "," + u128_str(m[2]) +
         "," + u128_str(m[3]);
    std::snprintf(b, sizeof b, " gmax=%" PRIu64 ":%" PRIu64 " gtail=", gmax_, gmax_lo_);
    o += b;
    if (tail_gaps_.empty()) o += "-";
    bool t1 = true;
    for (auto &t : tail_gaps_) {
        std::snprintf(b, sizeof b, "%s%u:%" PRIu64 ":%" PRIu64, t1 ? "" : ";", t.first, t.second.first,
                      t.second.second);
        o += b;
        t1 = false;
    }
    o += " ghist=" + dense_list(ghist_);
    return o;
}

std::string RunAccumulator::gbstats_line(const char *version) const
{
    // the reference's run line against an empty campaign: new_first lists
    // every first occurrence of the run's tail bins
    std::string l = gb::gbstats_line(record(true), std::vector<uint64_t>(GBC_NCAND, 0), version);
    if (!l.empty() && l.back() == '\n') l.pop_back();
    return l;
}

RunRecord RunAccumulator::record(bool gaps_on) const
{
    RunRecord r;
    r.start = start_;
    r.limit = limit_;
    r.evens = evens_;
    r.evens_sampled = evens_sampled_;
    r.tail_t = tail_t_;
    r.samp = samp_;
    r.tail_cls = tail_cls_;
    r.tail_agg = tail_agg_;
    r.first = first_tail_;
    r.beyond = beyond_list_;
    static const int u[8] = {1, 7, 11, 13, 17, 19, 23, 29};
    for (int i = 0; i < 8; ++i) r.primes30[i] = primes30_[u[i]];
    r.twins30[0] = twins30_[11];
    r.twins30[1] = twins30_[17];
    r.twins30[2] = twins30_[29];
    r.gaps_on = gaps_on;
    if (gaps_on) {
        // every segment is walked: the walk totals are the run's gaps (one
        // per prime of [start + 1, limit - 1], upper prime in that range)
        GapTotals &g = r.gaps;
        g.n = primes();
        g.wn = gap_count();
        g.wd[0] = g.wd[1] = g.wd[2] = g.wd[3] = odd_gaps_;
        for (size_t i = 0; i < ghist_.size(); ++i) {
            const u128 c = ghist_[i], gg = 2 * i, g2 = gg * gg;
            g.wd[0] += c * gg;
            g.wd[1] += c * g2;
            g.wd[2] += c * g2 * gg;
            g.wd[3] += c * g2 * g2;
        }
        g.d1 = g.wd[0];
        g.samp = ghist_;
        g.gmax = gmax_;
        g.gmax_lo = gmax_lo_;
        g.all_walked = true;
        g.tail = tail_gaps_;
        r.walk_evens = evens_;
    }
    return r;
}

std::vector<std::pair<uint64_t, uint64_t>> plan_segments(uint64_t start, uint64_t limit, uint64_t segment_even)
{
    std::vector<std::pair<uint64_t, uint64_t>> segs;
    uint64_t s = start;
    while (s <= limit) {
        uint64_t len = segment_even;
        // the lowest evens reach q < 7 and take the generic checker: keep
        // that segment short
        if (s < GBC_MAX_CAND + 7) len = std::min<uint64_t>(len, 65536);
        const uint64_t e = limit - s <= len - 2 ? limit : s + len - 2;
        segs.push_back({s, e});
        if (e >= limit) break;
        s = e + 2;
    }
    return segs;
}

namespace {

struct CtxCloser {
    void operator()(gbc_ctx *c) const { gbc_destroy(c); }
};

void check(gbc_ctx *ctx, int rc, const char *what)
{
    if (rc != GBC_OK) throw GbcError(rc, std::string(what) + ": " + gbc_last_error(ctx));
}

}  // namespace

RangeStats run_range(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t segment_even, uint32_t max_batch,
                     uint16_t *pn, RunAccumulator *acc_out, uint32_t sample_every, bool per_segment)
{
    RangeStats st;
    const auto t0 = std::chrono::steady_clock::now();
    if (start < 4) start = 4;
    if (start & 1) start += 1;
    limit &= ~uint64_t(1);
    if (limit < 6 || start > limit) throw GbcError(GBC_E_ARG, "no even n >= 4 in [start, limit] (need limit >= 6)");
    st.start = start;
    st.limit = limit;
    const auto segs = plan_segments(start, limit, segment_even);
    RunAccumulator acc(start, limit);
    std::vector<std::vector<std::pair<uint64_t, uint64_t>>> batches;
    std::vector<std::vector<uint32_t>> flags;
    for (size_t i = 0; i < segs.size(); i += max_batch) {
        batches.emplace_back(segs.begin() + i, segs.begin() + std::min(segs.size(), i + max_batch));
        std::vector<uint32_t> f;
        for (size_t j = i; j < std::min(segs.size(), i + max_batch); ++j)
            f.push_back(pn ? 0u : segment_flag(sample_every, j));
        flags.push_back(f);
    }
    std::vector<gbc_segment_result> out[2];
    double gpu_ms = 0;
    Outputs *outs = outputs_of(ctx);
    const std::vector<uint16_t> cand = outs ? candidates() : std::vector<uint16_t>();
    const uint64_t evens_total = (limit - start) / 2 + 1;
    auto t_last = std::chrono::steady_clock::now();
    auto collect = [&](size_t b) {
        const int slot = int(b & 1);
        const int n = int(batches[b].size());
        out[slot].resize(n);
        gbc_batch_times tm{};
        check(ctx, gbc_collect(ctx, slot, out[slot].data(), n, &tm, 600000), "collect");
        if (per_segment) {
            const auto now = std::chrono::steady_clock::now();
            const double wall = std::chrono::duration<double, std::milli>(now - t_last).count();
            t_last = now;
            uint64_t be = 0;
            for (int i = 0; i < n; ++i) be += out[slot][i].evens;
            for (int i = 0; i < n; ++i) {
                const auto &r = out[slot][i];
                const double f = double(r.evens) / double(be);
                st.per_segment.push_back({r.seg_start, r.seg_end, r.evens, r.nleft, tm.ms_tile * f, tm.ms_large * f,
                                          (tm.ms_check + tm.ms_count) * f, wall * f});
            }
        }
        gpu_ms += tm.ms_total;
        st.tile_ms += tm.ms_tile;
        st.large_ms += tm.ms_large;
        st.check_ms += tm.ms_check;
        st.count_ms += tm.ms_count;
        for (int i = 0; i < n; ++i) {
            acc.add_segment(out[slot][i]);
            if (outs) outs->add_segment(out[slot][i], cand);
            if (pn) {
                const auto &r = out[slot][i];
                check(ctx, gbc_copy_pn(ctx, slot, i, pn + (r.seg_start - start) / 2, r.evens), "copy p(n)");
            }
        }
        if (outs)
            outs->write_live(start, limit, acc.evens(), evens_total,
                             std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(), acc,
                             b + 1 == batches.size());
    };
    for (size_t b = 0; b < batches.size(); ++b) {
        std::vector<uint64_t> bounds;
        for (auto &s : batches[b]) {
            bounds.push_back(s.first);
            bounds.push_back(s.second);
        }
        check(ctx, gbc_enqueue_batch(ctx, int(b & 1), bounds.data(), flags[b].data(), int(batches[b].size()), limit),
              "enqueue");
        if (b) collect(b - 1);
    }
    collect(batches.size() - 1);
    st.evens = acc.evens();
    st.segments = segs.size();
    st.batches = batches.size();
    st.leftovers = acc.leftovers();
    st.pmax = acc.pmax();
    st.primes = acc.primes();
    st.twins = acc.twins();
    st.evens_sampled = acc.evens_sampled();
    st.tail_evens = acc.tail_evens();
    st.pending = acc.pending();
    st.gpu_seconds = gpu_ms / 1e3;
    st.wall_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    st.stats_line = acc.stats_ref_line();
    st.gbstats_line = acc.gbstats_line(kVersion);
    st.ridges = acc.ridges();
    // the passed run into the campaign state, once (GoldbachStats::commit)
    if (StatsCampaign *camp = campaign_of(ctx); camp && start >= kStatsMinStart) {
        std::string l = camp->commit(acc.record(stats_gaps_of(ctx)), &st.stats_committed);
        if (!l.empty() && l.back() == '\n') l.pop_back();
        st.gbstats_line = l;
    }
    if (outs) outs->finish_run();
    if (acc_out) *acc_out = acc;
    return st;
}

RangeStats run_sparse(uint64_t limit, bool verbose, uint64_t start_even, uint32_t dlt_log2)
{
    if (start_even < 4) start_even = 4;
    if (start_even & 1) ++start_even;
    if (limit & 1) --limit;
    if (start_even > limit) throw GbcError(GBC_E_ARG, "sparse: start > limit");
    gbc_sparse_config cfg{};
    cfg.limit = limit;
    cfg.dlt_log2 = dlt_log2;
    gbc_sparse *sp = nullptr;
    int rc = gbc_sparse_create(&cfg, &sp);
    const auto done = [&](int code, const char *what) {
        const std::string msg = std::string(what) + ": " + gbc_sparse_last_error(sp);
        gbc_sparse_destroy(sp);
        throw GbcError(code, msg);
    };
    if (rc != GBC_OK) done(rc, "gbc_sparse_create");
    gbc_sparse_result r{};
    rc = gbc_sparse_verify(sp, start_even, limit, &r);
    if (rc != GBC_OK) done(rc, "gbc_sparse_verify");
    gbc_sparse_destroy(sp);
    RangeStats st;
    st.start = start_even;
    st.limit = limit;
    st.evens = r.evens;
    st.segments = r.segments;
    st.batches = r.segments;
    st.leftovers = r.pending;
    st.gpu_seconds = (r.ms_sieve + r.ms_large + r.ms_check) / 1e3;
    st.wall_seconds = r.ms_total / 1e3;
    st.tile_ms = r.ms_sieve;
    st.large_ms = r.ms_large;
    st.check_ms = r.ms_check;
    if (verbose)
        std::fprintf(stderr, "sparse [%" PRIu64 ", %" PRIu64 "]: %" PRIu64 " segments, sieve %.3f large %.3f check "
                     "%.3f ms, %" PRIu64 " evens left to the CPU\n",
                     st.start, st.limit, st.segments, r.ms_sieve, r.ms_large, r.ms_check, r.pending);
    return st;
}

}  // namespace gb

extern "C" int gbc_verify_range(gbc_ctx *ctx, uint64_t start, uint64_t limit, gbc_run_result *res, char *line,
                                uint64_t line_cap, uint16_t *pn)
{
    if (!ctx) return GBC_E_ARG;
    try {
        gbc_config cfg{};
        if (gbc_get_config(ctx, &cfg) != GBC_OK) return GBC_E_ARG;
        gb::RangeStats st =
            gb::run_range(ctx, start, limit, cfg.segment_even, cfg.max_batch, pn, nullptr, cfg.sample_every);
        if (res) {
            res->start = st.start;
            res->limit = st.limit;
            res->evens = st.evens;
            res->segments = st.segments;
            res->batches = st.batches;
            res->leftovers = st.leftovers;
            res->pmax = st.pmax;
            res->primes = st.primes;
            res->twins = st.twins;
            res->gpu_seconds = st.gpu_seconds;
            res->wall_seconds = st.wall_seconds;
        }
        if (line && line_cap) {
            // the stats_ref line when every segment was sampled, else the GBSTATS v2 line
            const std::string &l = st.stats_line.empty() ? st.gbstats_line : st.stats_line;
            if (l.size() + 1 > line_cap) return GBC_E_OVERFLOW;
            std::memcpy(line, l.c_str(), l.size() + 1);
        }
        return GBC_OK;
    } catch (const gb::GbcError &e) {
        gbh_set_error(ctx, e.what());
        return e.code;
    } catch (const std::exception &e) {
        gbh_set_error(ctx, e.what());
        return GBC_E_DEVICE;
    }
}

extern "C" int gbc_set_stats(gbc_ctx *ctx, const char *state, const char *log, const char *version, int gaps)
{
    if (!ctx) return GBC_E_ARG;
    if (!state || !*state) {
        gbh_set_stats(ctx, nullptr, nullptr, true);
        return GBC_OK;
    }
    if (!log || !*log) {
        gbh_set_error(ctx, "gbc_set_stats: a state file needs a log file");
        return GBC_E_ARG;
    }
    try {
        auto *c = new gb::StatsCampaign(state, log, version && *version ? version : gb::kVersion);
        try {
            c->check();
        } catch (...) {
            delete c;
            throw;
        }
        gbh_set_stats(ctx, c, [](void *p) { delete static_cast<gb::StatsCampaign *>(p); }, gaps != 0);
        return GBC_OK;
    } catch (const std::exception &e) {
        gbh_set_error(ctx, e.what());
        return GBC_E_STATE;
    }
}

extern "C" int gbc_stats_commit(const char *state, const char *log, const char *version, int gaps, uint64_t start,
                                uint64_t limit, const gbc_segment_result *segs, int nseg, char *line, uint64_t line_cap,
                                int *merged, char *err, size_t err_cap)
{
    const auto fail = [&](int code, const std::string &m) {
        if (err && err_cap) std::snprintf(err, err_cap, "%s", m.c_str());
        return code;
    };
    if (!state || !*state || !log || !*log || !segs || nseg < 1 || start < gb::kStatsMinStart || (start & 1) ||
        (limit & 1) || limit < start)
        return fail(GBC_E_ARG, "need state and log paths, results, and even start >= 1e6 <= even limit");
    uint64_t next = start;
    for (int i = 0; i < nseg; ++i) {
        if (segs[i].seg_start != next || segs[i].seg_end < segs[i].seg_start ||
            segs[i].evens != (segs[i].seg_end - segs[i].seg_start) / 2 + 1)
            return fail(GBC_E_ARG, "the segments must cover [start, limit] in order");
        next = segs[i].seg_end + 2;
    }
    if (next != limit + 2) return fail(GBC_E_ARG, "the segments must cover [start, limit] in order");
    try {
        gb::RunAccumulator acc(start, limit);
        for (int i = 0; i < nseg; ++i) acc.add_segment(segs[i]);
        gb::StatsCampaign camp(state, log, version && *version ? version : gb::kVersion);
        bool m = false;
        std::string l = camp.commit(acc.record(gaps != 0), &m);
        if (!l.empty() && l.back() == '\n') l.pop_back();
        if (merged) *merged = m ? 1 : 0;
        if (line && line_cap) {
            if (l.size() + 1 > line_cap) return fail(GBC_E_OVERFLOW, "line buffer too small");
            std::memcpy(line, l.c_str(), l.size() + 1);
        }
        return GBC_OK;
    } catch (const std::exception &e) {
        return fail(GBC_E_STATE, e.what());
    }
}
