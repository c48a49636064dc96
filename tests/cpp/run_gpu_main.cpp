// run_gpu_main.cpp -- a caller of the reference's C++ interface, compiled
// against include/gb_verifier.hpp and linked with libgbc.so: what the
// reference's src/main.cpp does with gb::run_gpu (src/main.cpp:356-361),
// with the RunStats fields printed as key=value lines for the tests.
//
// usage: run_gpu_main LIMIT SEGMENT START COLLECT   (verify [START, LIMIT])
//        run_gpu_main --device-info | --cpu-check LIMIT
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>

#include "gb_verifier.hpp"

int main(int argc, char **argv)
{
    try {
        if (argc == 2 && !std::strcmp(argv[1], "--device-info")) {
            gb::print_device_info();
            return 0;
        }
        if (argc == 3 && !std::strcmp(argv[1], "--cpu-check"))
            return gb::verify_cpu(std::strtoull(argv[2], nullptr, 10), false) ? 0 : 1;
        if (argc != 5) return 2;
        const uint64_t limit = std::strtoull(argv[1], nullptr, 10), seg = std::strtoull(argv[2], nullptr, 10);
        const uint64_t start = std::strtoull(argv[3], nullptr, 10);
        const bool collect = std::atoi(argv[4]) != 0;
        const gb::RunStats s = gb::run_gpu(limit, seg, "goldbach.spv", false, start, 0, nullptr, collect);
        std::printf("limit=%" PRIu64 "\nstart=%" PRIu64 "\nsegments=%" PRIu64 "\nleftovers=%" PRIu64 "\n", s.limit,
                    s.start, s.segments, s.leftovers);
        std::printf("gpu_seconds=%.6f\nevens_per_second=%.6g\nsieve_seconds=%.6f\nverify_seconds=%.6f\n", s.gpu_seconds,
                    s.evens_per_second, s.sieve_seconds, s.verify_seconds);
        std::printf("split_used=%u\ntotal_tiles=%" PRIu64 "\nridge_min=%u\nridge_top=%zu\n", s.split_used, s.total_tiles,
                    s.ridge_min, s.ridge_top.size());
        std::printf("stats_on=%d\nstats_pmax=%" PRIu64 "\nstats_primes=%" PRIu64 "\nstats_twins=%" PRIu64
                    "\nstats_sampled=%" PRIu64 "\nstats_tail=%" PRIu64 "\n",
                    int(s.stats_on), s.stats_pmax, s.stats_primes, s.stats_twins, s.stats_sampled, s.stats_tail);
        uint64_t ev = 0;
        for (const auto &r : s.per_segment) ev += r.evens;
        std::printf("per_segment=%zu\nper_segment_evens=%" PRIu64 "\n", s.per_segment.size(), ev);
        for (const auto &r : s.ridge_top)
            std::printf("ridge=%" PRIu64 ":%" PRIu64 ":%" PRIu64 "\n", r.n, r.p, r.q);
        return 0;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "FAIL: %s\n", e.what());
        return 1;
    }
}
