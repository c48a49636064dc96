// abi_probe.cpp -- the binary interface of the C++ entry points: prints the
// layout of RunStats, SegmentStats and RidgeEntry (offset and size of every
// member) and, compiled with -DNAME_CALLS, references every entry point so
// the object file's undefined symbols are their mangled names. Built once
// against the reference's include/verifier.hpp + include/sparse_run.hpp
// (-DREF_HEADERS: tests/golden/make_abi_golden.py writes the fixture) and
// once against include/gb_verifier.hpp (tests/test_verifier_abi.py).
#include <cstddef>
#include <cstdio>
#ifdef REF_HEADERS
#include "sparse_run.hpp"
#include "verifier.hpp"
#else
#include "gb_verifier.hpp"
#endif

#define F(T, m) std::printf("layout %s.%s %zu %zu\n", #T, #m, offsetof(gb::T, m), sizeof(((gb::T *)nullptr)->m))

int main(int argc, char **)
{
    std::printf("size RunStats %zu %zu\n", sizeof(gb::RunStats), alignof(gb::RunStats));
    std::printf("size SegmentStats %zu %zu\n", sizeof(gb::SegmentStats), alignof(gb::SegmentStats));
    std::printf("size RidgeEntry %zu %zu\n", sizeof(gb::RidgeEntry), alignof(gb::RidgeEntry));
    F(RidgeEntry, n); F(RidgeEntry, p); F(RidgeEntry, q); F(RidgeEntry, seg); F(RidgeEntry, found);
    F(SegmentStats, seg_start); F(SegmentStats, seg_end); F(SegmentStats, evens); F(SegmentStats, tiles);
    F(SegmentStats, large_items); F(SegmentStats, sieve_split); F(SegmentStats, mask_count);
    F(SegmentStats, leftovers); F(SegmentStats, sieve_seconds); F(SegmentStats, large_seconds);
    F(SegmentStats, check_seconds); F(SegmentStats, offset_seconds); F(SegmentStats, wall_seconds);
    F(RunStats, limit); F(RunStats, start); F(RunStats, segment_used); F(RunStats, segments); F(RunStats, leftovers);
    F(RunStats, init_seconds); F(RunStats, init_cache_s); F(RunStats, init_module_s); F(RunStats, init_upload_s);
    F(RunStats, gpu_seconds); F(RunStats, total_seconds); F(RunStats, evens_per_second); F(RunStats, sieve_seconds);
    F(RunStats, large_seconds); F(RunStats, verify_seconds); F(RunStats, sync_seconds); F(RunStats, offset_seconds);
    F(RunStats, table_seconds); F(RunStats, total_tiles); F(RunStats, total_large_items); F(RunStats, split_used);
    F(RunStats, ridge_min); F(RunStats, ridge_found); F(RunStats, ridge_dropped); F(RunStats, ridge_top);
    F(RunStats, stats_on); F(RunStats, stats_pmax); F(RunStats, stats_primes); F(RunStats, stats_twins);
    F(RunStats, stats_sampled); F(RunStats, stats_tail); F(RunStats, per_segment);
#ifdef NAME_CALLS
    if (argc > 1000) {  // never true: only names the entry points
        gb::RunStats s = gb::run_gpu(0, 0, std::string(), false);
        s = gb::run_gpu(0, 0, std::string(), false, 4, 0, nullptr, false);
        gb::print_device_info();
        (void)gb::verify_cpu(0, false);
        s = gb::run_gpu_sparse(0, 0, std::string(), false, 0, 0, nullptr, false);
        return int(s.segments);
    }
#endif
    (void)argc;
    return 0;
}
