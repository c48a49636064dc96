// gb_journal.cpp -- the slice runner and its journal (the reference's
// tools/run_range.sh contract, docs/PIPELINE.md:12-24, 114-122):
//   resume   walk the journal's PASS chain from the range's start: the next
//            slice starts 2 after the last contiguous PASS slice's end;
//            RETRY rows and PASS rows off the chain are ignored
//   slices   [a, min(a + slice - 2, limit)], verified one after another on
//            one resident context (the reference starts a process per slice)
//   rows     "PASS a b ts <csv> release=R" per slice (" attempts=2" when it
//            passed on the retry), "RETRY a b ts reason=..." for a failed
//            first attempt; a slice that fails twice stops the run
//   stop     a stop file present before a slice ends the run cleanly with
//            the resume point intact
#include <sys/stat.h>

#include <cerrno>
#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <functional>
#include <map>
#include <sstream>
#include <string>

#include "gb_run.hpp"

void gbh_set_error(gbc_ctx *ctx, const char *msg);  // gbc_api.cu

namespace gb {

namespace {

std::string utc_now()
{
    const std::time_t t = std::time(nullptr);
    std::tm tm{};
    gmtime_r(&t, &tm);
    char b[32];
    std::strftime(b, sizeof b, "%Y-%m-%dT%H:%M:%SZ", &tm);
    return b;
}

bool file_exists(const char *p)
{
    struct stat st;
    return p && *p && stat(p, &st) == 0;
}

}  // namespace

// The reference's --csv line for a run (src/main.cpp:191-215): key=value
// pairs, the keys this path has in common with it.
std::string csv_line(const RangeStats &st, uint64_t segment)
{
    const double eps = st.gpu_seconds > 0 ? double(st.evens) / st.gpu_seconds : 0.0;
    const uint64_t ridge_max = st.ridges.empty() ? 0 : st.ridges.front().p;
    char b[1024];
    std::snprintf(b, sizeof b,
                  "version=gb300-1.0 limit=%" PRIu64 " start=%" PRIu64 " segment=%" PRIu64 " split=0 segments=%" PRIu64
                  " leftovers=%" PRIu64 " result=PASS gpu_s=%.4f total_s=%.4f sieve_s=%.4f large_s=%.4f check_s=%.4f"
                  " count_s=%.4f evens_per_sec=%.6g ridge_min=%u ridge_found=%zu ridge_max=%" PRIu64
                  " stats=1 stats_tail=%" PRIu64 " stats_sampled=%" PRIu64 " stats_pmax=%" PRIu64 " primes=%" PRIu64
                  " twins=%" PRIu64,
                  st.limit, st.start, segment, st.segments, st.leftovers, st.gpu_seconds, st.wall_seconds,
                  st.tile_ms / 1e3, st.large_ms / 1e3, st.check_ms / 1e3, st.count_ms / 1e3, eps, GBC_TAIL_T,
                  st.ridges.size(), ridge_max, st.tail_evens, st.evens_sampled, st.pmax, st.primes, st.twins);
    return b;
}

// The resume point of [start, ...] in a journal: start, moved past every
// PASS slice that continues the chain.
uint64_t journal_resume(const std::string &path, uint64_t start)
{
    std::ifstream in(path);
    std::map<uint64_t, uint64_t> pass;  // a -> b of the PASS rows
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string tag;
        uint64_t a = 0, b = 0;
        if (!(ss >> tag) || tag != "PASS" || !(ss >> a >> b) || b < a) continue;
        auto &slot = pass[a];
        if (b > slot) slot = b;
    }
    uint64_t next = start;
    for (;;) {
        auto it = pass.find(next);
        if (it == pass.end()) break;
        next = it->second + 2;
    }
    return next;
}

namespace {

// The journaled slice loop over [start, limit]: verify(a, b) verifies one
// slice and returns its csv line, or throws GbcError.
uint64_t journal_loop(uint64_t start, uint64_t limit, uint64_t slice, const std::string &journal,
                      const std::string &release, const char *stop_file, FILE *log, int *stopped,
                      const std::function<std::string(uint64_t, uint64_t)> &verify)
{
    if (stopped) *stopped = 0;
    uint64_t next = journal_resume(journal, start), done = 0;
    if (log)
        std::fprintf(log, "%s %s [%" PRIu64 ", %" PRIu64 "] slice %" PRIu64 " from %" PRIu64 "\n", utc_now().c_str(),
                     next == start ? "start" : "resume", start, limit, slice, next);
    const auto t0 = std::chrono::steady_clock::now();
    while (next <= limit) {
        if (file_exists(stop_file)) {
            if (log) std::fprintf(log, "%s stop file: resume point %" PRIu64 "\n", utc_now().c_str(), next);
            if (stopped) *stopped = 1;
            return done;
        }
        const uint64_t a = next, b = limit - a < slice - 2 ? limit : a + slice - 2;
        std::string csv;
        int attempts = 0;
        for (;;) {
            ++attempts;
            try {
                csv = verify(a, b);
                break;
            } catch (const GbcError &e) {
                if (attempts == 1)
                    std::ofstream(journal, std::ios::app)
                        << "RETRY " << a << ' ' << b << ' ' << utc_now() << " reason=" << e.code << '\n';
                if (log) std::fprintf(log, "%s FAILED [%" PRIu64 ", %" PRIu64 "]: %s\n", utc_now().c_str(), a, b, e.what());
                if (attempts == 2) {
                    if (log) std::fprintf(log, "%s STOPPED: [%" PRIu64 ", %" PRIu64 "] failed twice\n",
                                          utc_now().c_str(), a, b);
                    throw;
                }
            }
        }
        {
            std::ofstream out(journal, std::ios::app);
            out << "PASS " << a << ' ' << b << ' ' << utc_now() << ' ' << csv << " release=" << release
                << (attempts == 2 ? " attempts=2" : "") << '\n';
            if (!out) throw GbcError(GBC_E_ARG, "cannot append to the journal " + journal);
        }
        ++done;
        next = b + 2;
        if (log) {
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            const double frac = double(next - start) / double(limit - start + 2);
            std::fprintf(log, "%s PASS [%" PRIu64 ", %" PRIu64 "] %.2f%% done, %.1f s left\n", utc_now().c_str(), a, b,
                         100.0 * frac, frac > 0 ? el * (1 - frac) / frac : 0.0);
        }
    }
    if (log) std::fprintf(log, "%s COMPLETE [%" PRIu64 ", %" PRIu64 "]\n", utc_now().c_str(), start, limit);
    return done;
}

}  // namespace

// Runs [start, limit] in journaled slices on ctx. Returns the number of
// slices verified now; *stopped = 1 when the stop file ended the run early.
// Throws GbcError when a slice fails twice (the journal then holds its RETRY
// row and the resume point is that slice).
uint64_t run_slices(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t slice, const std::string &journal,
                    const std::string &release, const char *stop_file, FILE *log, int *stopped)
{
    if (slice < 4 || (slice & 1)) throw GbcError(GBC_E_ARG, "slice must be even and at least 4");
    if (start & 1) ++start;
    limit &= ~uint64_t(1);
    gbc_config cfg{};
    if (gbc_get_config(ctx, &cfg) != GBC_OK) throw GbcError(GBC_E_ARG, "no context");
    if (limit > cfg.limit) throw GbcError(GBC_E_ARG, "limit above the context's limit");
    return journal_loop(start, limit, slice, journal, release, stop_file, log, stopped, [&](uint64_t a, uint64_t b) {
        const RangeStats st = run_range(ctx, a, b, cfg.segment_even, cfg.max_batch, nullptr, nullptr, cfg.sample_every);
        return csv_line(st, cfg.segment_even);
    });
}

// The sparse cross-check's csv line (the keys it shares with the dense
// line; path=sparse, no statistics).
std::string sparse_csv_line(const RangeStats &st)
{
    const double eps = st.gpu_seconds > 0 ? double(st.evens) / st.gpu_seconds : 0.0;
    char b[512];
    std::snprintf(b, sizeof b,
                  "version=gb300-1.0 path=sparse limit=%" PRIu64 " start=%" PRIu64 " segments=%" PRIu64
                  " leftovers=%" PRIu64 " result=PASS gpu_s=%.4f total_s=%.4f sieve_s=%.4f large_s=%.4f check_s=%.4f"
                  " evens_per_sec=%.6g stats=0",
                  st.limit, st.start, st.segments, st.leftovers, st.gpu_seconds, st.wall_seconds, st.tile_ms / 1e3,
                  st.large_ms / 1e3, st.check_ms / 1e3, eps);
    return b;
}

// The sparse cross-check of [start, limit] in journaled slices on sp
// (ci/sparse_crosscheck.sh run: run_range with GB_SPARSE=1 and its own
// journal): the same rows, resume rule and stop file as run_slices.
uint64_t run_sparse_slices(gbc_sparse *sp, uint64_t start, uint64_t limit, uint64_t slice, const std::string &journal,
                           const std::string &release, const char *stop_file, FILE *log, int *stopped)
{
    if (slice < 4 || (slice & 1)) throw GbcError(GBC_E_ARG, "slice must be even and at least 4");
    if (start & 1) ++start;
    limit &= ~uint64_t(1);
    return journal_loop(start, limit, slice, journal, release, stop_file, log, stopped, [&](uint64_t a, uint64_t b) {
        gbc_sparse_result r{};
        const int rc = gbc_sparse_verify(sp, a, b, &r);
        if (rc != GBC_OK) throw GbcError(rc, std::string("gbc_sparse_verify: ") + gbc_sparse_last_error(sp));
        RangeStats st;
        st.start = a;
        st.limit = b;
        st.evens = r.evens;
        st.segments = r.segments;
        st.leftovers = r.pending;
        st.gpu_seconds = (r.ms_sieve + r.ms_large + r.ms_check) / 1e3;
        st.wall_seconds = r.ms_total / 1e3;
        st.tile_ms = r.ms_sieve;
        st.large_ms = r.ms_large;
        st.check_ms = r.ms_check;
        return sparse_csv_line(st);
    });
}

}  // namespace gb

extern "C" int gbc_journal_resume(const char *path, uint64_t start, uint64_t *next)
{
    if (!path || !next) return GBC_E_ARG;
    *next = gb::journal_resume(path, start);
    return GBC_OK;
}

extern "C" int gbc_run_slices(gbc_ctx *ctx, uint64_t start, uint64_t limit, uint64_t slice, const char *journal,
                              const char *release, const char *stop_file, uint64_t *slices_done, int *stopped)
{
    if (!ctx || !journal) return GBC_E_ARG;
    try {
        const uint64_t n = gb::run_slices(ctx, start, limit, slice, journal, release ? release : "gb300-1.0",
                                          stop_file, nullptr, stopped);
        if (slices_done) *slices_done = n;
        return GBC_OK;
    } catch (const gb::GbcError &e) {
        gbh_set_error(ctx, e.what());
        return e.code;
    } catch (const std::exception &e) {
        gbh_set_error(ctx, e.what());
        return GBC_E_DEVICE;
    }
}

extern "C" int gbc_sparse_run_slices(gbc_sparse *sp, uint64_t start, uint64_t limit, uint64_t slice,
                                     const char *journal, const char *release, const char *stop_file,
                                     uint64_t *slices_done, int *stopped)
{
    if (!sp || !journal) return GBC_E_ARG;
    try {
        const uint64_t n = gb::run_sparse_slices(sp, start, limit, slice, journal, release ? release : "gb300-1.0",
                                                 stop_file, nullptr, stopped);
        if (slices_done) *slices_done = n;
        return GBC_OK;
    } catch (const gb::GbcError &e) {
        return e.code;
    } catch (const std::exception &) {
        return GBC_E_DEVICE;
    }
}
