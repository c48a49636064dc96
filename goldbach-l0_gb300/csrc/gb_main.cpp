// gb_main.cpp -- goldbach_gb300: command-line front end of the GB300 dense
// verify path. Flags and exit codes follow the reference's CLI
// (src/main.cpp:28-86, 265-411): --start, --limit (decimal or e-notation,
// strict), --segment, --csv; exit 0 = PASS, 1 = verification or GPU
// failure, 2 = usage error. --batch sets the segments per sieve batch;
// --stats prints the run's stats_ref line (tests/stats_ref.cpp:97-189).
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "gb_run.hpp"

namespace {

// Strict count parser: digits, or <digits>[.<digits>]e<digits> that is an
// exact integer (the reference's parse_count, src/main.cpp:28-57).
bool parse_count(const char *s, uint64_t &out)
{
    if (!s || !*s) return false;
    const char *e = std::strchr(s, 'e');
    if (!e) e = std::strchr(s, 'E');
    if (!e) {
        uint64_t v = 0;
        for (const char *p = s; *p; ++p) {
            if (*p < '0' || *p > '9') return false;
            const uint64_t d = uint64_t(*p - '0');
            if (v > (UINT64_MAX - d) / 10) return false;
            v = v * 10 + d;
        }
        out = v;
        return true;
    }
    // mantissa digits with an optional point, exponent digits
    std::string mant(s, e), digits;
    int frac = 0;
    bool point = false;
    for (char c : mant) {
        if (c == '.') {
            if (point) return false;
            point = true;
        } else if (c >= '0' && c <= '9') {
            digits += c;
            if (point) ++frac;
        } else return false;
    }
    if (digits.empty()) return false;
    int ex = 0;
    const char *x = e + 1;
    if (!*x) return false;
    for (; *x; ++x) {
        if (*x < '0' || *x > '9' || ex > 40) return false;
        ex = ex * 10 + (*x - '0');
    }
    ex -= frac;
    if (ex < 0) return false;
    uint64_t v = 0;
    for (char c : digits) {
        const uint64_t d = uint64_t(c - '0');
        if (v > (UINT64_MAX - d) / 10) return false;
        v = v * 10 + d;
    }
    for (int i = 0; i < ex; ++i) {
        if (v > UINT64_MAX / 10) return false;
        v *= 10;
    }
    out = v;
    return true;
}

int usage()
{
    std::fprintf(stderr,
                 "usage: goldbach_gb300 [--start N] --limit N [--segment N] [--batch N] [--stats-sample N] [--csv] "
                 "[--stats] [--verbose]\n"
                 "       goldbach_gb300 --start N --limit N --sparse [--csv] [--verbose]   (the sparse class map "
                 "cross-check; start well above sqrt(limit))\n"
                 "       goldbach_gb300 --start N --limit N --sparse --slice N --journal FILE [--release ID] "
                 "[--stop-file F]   (journaled cross-check)\n"
                 "       goldbach_gb300 --start N --limit N --crosscheck-status DENSE_JOURNAL SPARSE_JOURNAL\n"
                 "       goldbach_gb300 --start N --limit N --slice N --journal FILE [--release ID] [--stop-file F]\n"
                 "                      [--segment N] [--batch N] [--stats-sample N]   (journaled slices; exit 3 "
                 "on the stop file)\n");
    return 2;
}

}  // namespace

int main(int argc, char **argv)
{
    uint64_t start = 4, limit = 0, segment = GBC_DEFAULT_SEGMENT, batch = 8, sample = 1, slice = 0;
    bool csv = false, stats = false, verbose = false, sparse = false;
    std::string journal, release = "gb300-1.0", stop_file, status_dense, status_sparse;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto val = [&](uint64_t &dst) {
            if (i + 1 >= argc || !parse_count(argv[i + 1], dst)) return false;
            ++i;
            return true;
        };
        if (a == "--start") {
            if (!val(start)) return usage();
        } else if (a == "--limit") {
            if (!val(limit)) return usage();
        } else if (a == "--segment") {
            if (!val(segment)) return usage();
        } else if (a == "--batch") {
            if (!val(batch) || !batch || batch > 256) return usage();
        } else if (a == "--stats-sample") {
            if (!val(sample) || !sample || sample > (1u << 30)) return usage();
        } else if (a == "--slice") {
            if (!val(slice) || slice < 4 || (slice & 1)) return usage();
        } else if (a == "--journal" || a == "--release" || a == "--stop-file") {
            if (i + 1 >= argc) return usage();
            (a == "--journal" ? journal : a == "--release" ? release : stop_file) = argv[++i];
        } else if (a == "--csv") csv = true;
        else if (a == "--stats") stats = true;
        else if (a == "--verbose") verbose = true;
        else if (a == "--sparse") sparse = true;
        else if (a == "--crosscheck-status") {
            if (i + 2 >= argc) return usage();
            status_dense = argv[++i];
            status_sparse = argv[++i];
        } else return usage();
    }
    if (!limit) return usage();
    if (start > limit) {
        std::fprintf(stderr, "empty range: start %" PRIu64 " > limit %" PRIu64 "\n", start, limit);
        return 2;
    }
    if (limit > GBC_MAX_LIMIT) {
        std::fprintf(stderr, "limit %" PRIu64 " is above the supported maximum 2^64 - 2^40\n", limit);
        return 1;
    }
    if ((slice != 0) != !journal.empty()) return usage();
    if (!status_dense.empty()) {
        // ci/sparse_crosscheck.sh status: the contiguous coverage of both
        // journals from start and the evens both have verified
        start += start & 1;
        const uint64_t d = gb::journal_resume(status_dense, start) - 2, s = gb::journal_resume(status_sparse, start) - 2;
        const uint64_t both = d < s ? d : s;
        std::printf("dense  (%s): verified [%" PRIu64 ", %" PRIu64 "]\n", status_dense.c_str(), start, d);
        std::printf("sparse (%s): verified [%" PRIu64 ", %" PRIu64 "]\n", status_sparse.c_str(), start, s);
        if (both + 2 > start)
            std::printf("both:   [%" PRIu64 ", %" PRIu64 "] = %" PRIu64 " evens, %.3f%% of [%" PRIu64 ", %" PRIu64 "]\n",
                        start, both, (both - start) / 2 + 1, 100.0 * double(both - start + 2) / double(limit - start + 2),
                        start, limit);
        else
            std::printf("both:   nothing yet\n");
        return 0;
    }
    if (sparse) {
        if (stats) return usage();
        if (slice) {
            gbc_sparse_config scfg{};
            scfg.limit = limit & ~uint64_t(1);
            gbc_sparse *sp = nullptr;
            int rc = gbc_sparse_create(&scfg, &sp);
            if (rc != GBC_OK) {
                std::fprintf(stderr, "FAIL: gbc_sparse_create: %s\n", gbc_sparse_last_error(sp));
                gbc_sparse_destroy(sp);
                return rc == GBC_E_ARG ? 2 : 1;
            }
            int code = 0;
            try {
                int stopped = 0;
                gb::run_sparse_slices(sp, start, limit, slice, journal, release,
                                      stop_file.empty() ? nullptr : stop_file.c_str(), stdout, &stopped);
                code = stopped ? 3 : 0;
            } catch (const gb::GbcError &e) {
                std::fprintf(stderr, "FAIL: %s\n", e.what());
                code = e.code == GBC_E_ARG ? 2 : 1;
            }
            gbc_sparse_destroy(sp);
            return code;
        }
        try {
            const gb::RangeStats st = gb::run_sparse(limit, verbose, start);
            const double eps = st.gpu_seconds > 0 ? double(st.evens) / st.gpu_seconds : 0.0;
            if (csv)
                std::printf("result=PASS,path=sparse,start=%" PRIu64 ",limit=%" PRIu64 ",evens=%" PRIu64
                            ",segments=%" PRIu64 ",leftovers=%" PRIu64 ",gpu_s=%.6f,wall_s=%.6f,evens_per_s=%.6g\n",
                            st.start, st.limit, st.evens, st.segments, st.leftovers, st.gpu_seconds, st.wall_seconds,
                            eps);
            else
                std::printf("PASS (sparse): every even n in [%" PRIu64 ", %" PRIu64 "] is a sum of two primes "
                            "(%" PRIu64 " evens, %" PRIu64 " segments, %" PRIu64 " leftovers, %.3f G evens/s)\n",
                            st.start, st.limit, st.evens, st.segments, st.leftovers, eps / 1e9);
            return 0;
        } catch (const gb::GbcError &e) {
            std::fprintf(stderr, "FAIL: %s\n", e.what());
            return e.code == GBC_E_ARG ? 2 : 1;
        }
    }
    gbc_config cfg{};
    cfg.limit = limit & ~uint64_t(1);
    cfg.segment_even = segment;
    cfg.max_batch = uint32_t(batch);
    cfg.sample_every = uint32_t(sample);
    gbc_ctx *ctx = nullptr;
    const int rc = gbc_create(&cfg, &ctx);
    if (rc != GBC_OK) {
        std::fprintf(stderr, "FAIL: gbc_create: %s\n", gbc_last_error(ctx));
        gbc_destroy(ctx);
        return rc == GBC_E_ARG ? 2 : 1;
    }
    gb::attach_env_outputs(ctx);
    if (slice) {
        int code = 0;
        try {
            int stopped = 0;
            gb::run_slices(ctx, start, limit, slice, journal, release, stop_file.empty() ? nullptr : stop_file.c_str(),
                           stdout, &stopped);
            code = stopped ? 3 : 0;
        } catch (const gb::GbcError &e) {
            std::fprintf(stderr, "FAIL: %s\n", e.what());
            code = e.code == GBC_E_ARG ? 2 : 1;
        }
        gbc_destroy(ctx);
        return code;
    }
    int code = 0;
    try {
        gbc_get_config(ctx, &cfg);
        const gb::RangeStats st = gb::run_range(ctx, start, limit, cfg.segment_even, cfg.max_batch, nullptr, nullptr,
                                              cfg.sample_every);
        if (verbose)
            std::fprintf(stderr, "run [%" PRIu64 ", %" PRIu64 "]: %" PRIu64 " segments, gpu %.3f s, wall %.3f s\n",
                         st.start, st.limit, st.segments, st.gpu_seconds, st.wall_seconds);
        const double eps = st.gpu_seconds > 0 ? double(st.evens) / st.gpu_seconds : 0.0;
        if (csv)
            std::printf("%s\n", gb::csv_line(st, cfg.segment_even).c_str());
        else
            std::printf("PASS: every even n in [%" PRIu64 ", %" PRIu64 "] is a sum of two primes "
                        "(%" PRIu64 " evens, largest p(n) %" PRIu64 ", %.3f G evens/s)\n",
                        st.start, st.limit, st.evens, st.pmax, eps / 1e9);
        if (stats) {
            std::printf("%s\n", st.gbstats_line.c_str());
            if (!st.stats_line.empty()) std::printf("%s\n", st.stats_line.c_str());
        }
    } catch (const gb::GbcError &e) {
        std::fprintf(stderr, "FAIL: %s\n", e.what());
        code = e.code == GBC_E_ARG ? 2 : 1;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "FAIL: %s\n", e.what());
        code = 1;
    }
    gbc_destroy(ctx);
    return code;
}
