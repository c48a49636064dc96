// gb_verifier.hpp -- the reference's C++ entry points of the dense and sparse
// verify paths, implemented by libgbc.so on one GB300.
//
// A drop-in for the reference's src/verifier.cpp and src/sparse.cpp: these
// declarations and structs are the reference's own interface (names, member
// order and types, default arguments), so code compiled against the
// reference's include/verifier.hpp, include/ridge.hpp (RidgeEntry) and
// include/sparse_run.hpp (run_gpu_sparse) links against libgbc.so instead of
// those objects with no source change. They have to be alike: the mangled
// names and the struct layouts are the binary interface.
//   include/verifier.hpp:12-28   SegmentStats
//   include/verifier.hpp:31-69   RunStats
//   include/verifier.hpp:71-125  run_gpu, print_device_info, verify_cpu
//   include/ridge.hpp:49-56      RidgeEntry
//   include/sparse_run.hpp:120-134 run_gpu_sparse
// What the arguments mean on this implementation is in gb_verifier.cpp's
// comments: the Level Zero module path and the prime cache path are
// accepted and not used (the kernels are compiled in; the sieving primes are
// computed in memory), and every knob the reference reads from its GB_*
// environment is read the same way.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace gb {

/// One tracked ridge: even n = p + q with p the smallest witness prime.
struct RidgeEntry {
    uint64_t n = 0;      // the even number
    uint64_t p = 0;      // the ridge: smallest prime of the partition
    uint64_t q = 0;      // n - p (prime)
    uint64_t seg = 0;    // segment start of the run that found it
    uint64_t found = 0;  // Unix time it first entered the store (0 = unknown)
};

// Per-segment measurements (populated when collect_segments is set).
struct SegmentStats {
    uint64_t seg_start      = 0;   // first even n of the segment
    uint64_t seg_end        = 0;   // last even n of the segment (inclusive)
    uint64_t evens          = 0;
    uint64_t tiles          = 0;   // shared-memory tiles of the segment's span (8 class arrays)
    uint64_t large_items    = 0;   // large-prime and hit-list primes that reach the segment
    uint32_t sieve_split    = 0;   // tile-sieve primes (odd primes up to the split)
    uint32_t mask_count     = 0;   // primes cleared by the whole-word patterns (7..67)
    uint32_t leftovers      = 0;   // evens without a witness <= 9781 in this segment
    double   sieve_seconds  = 0;   // the segment's share of its batch's sieve time (device events)
    double   large_seconds  = 0;   // ... of the large-prime and hit-list time
    double   check_seconds  = 0;   // ... of the checker time
    double   offset_seconds = 0;   // host offset preparation (none: 0)
    double   wall_seconds   = 0;   // the segment's share of its batch's wall time
};

// Totals and settings of one run (dense or sparse path).
struct RunStats {
    uint64_t limit            = 0;
    uint64_t start            = 0;
    uint64_t segment_used     = 0;   // segment span actually used when it differs from the argument
    uint64_t segments         = 0;
    uint64_t leftovers        = 0;   // evens without a witness <= 9781 (resolved on the GPU)
    double   init_seconds     = 0.0; // context: primes, tables, device buffers, multiplier table
    double   init_cache_s     = 0.0; // the context's creation (sieving primes, tables, slots)
    double   init_module_s    = 0.0; // no module to load: 0
    double   init_upload_s    = 0.0; // the prime-multiplier table build for the run
    double   gpu_seconds      = 0.0; // segment loop (wall)
    double   total_seconds    = 0.0;
    double   evens_per_second = 0.0;
    double   sieve_seconds    = 0.0; // device time of the tile sieve
    double   large_seconds    = 0.0; // device time of the large-prime and hit-list stages
    double   verify_seconds   = 0.0; // device time of the checkers
    double   sync_seconds     = 0.0; // loop wall time not in those stages
    double   offset_seconds   = 0.0; // host offset preparation (none: 0)
    double   table_seconds   = 0.0;  // host per-tile table build (none: 0)
    uint64_t total_tiles      = 0;
    uint64_t total_large_items = 0;
    uint32_t split_used       = 0;   // tile-sieve primes in force
    uint32_t ridge_min    = 0;
    uint64_t ridge_found  = 0;
    uint64_t ridge_dropped = 0;
    std::vector<RidgeEntry> ridge_top;
    bool     stats_on     = false;
    uint64_t stats_pmax   = 0;
    uint64_t stats_primes = 0;
    uint64_t stats_twins  = 0;
    uint64_t stats_sampled = 0;
    uint64_t stats_tail   = 0;
    std::vector<SegmentStats> per_segment;
};

/// Verifies Goldbach for every even n in [max(start_even, 4) rounded up to
/// even, limit] on the GPU and returns the run's timings, counters and exact
/// statistics. Throws std::runtime_error on any failure (nothing is
/// reported as passed then).
RunStats run_gpu(uint64_t limit,
                 uint64_t segment_even,
                 const std::string& spv_path,
                 bool verbose,
                 uint64_t start_even = 4,
                 uint32_t sieve_split_arg = 0,
                 const char* prime_cache_path = nullptr,
                 bool collect_segments = false);

/// Prints device / driver / runtime information and the build's tuning
/// constants to stdout, one block per GPU. Throws std::runtime_error when no
/// GPU is reported.
void print_device_info();

/// Independent CPU check by trial division (no GPU, no sieve), for small
/// limits: true when every even n in [4, limit] has a Goldbach partition.
bool verify_cpu(uint64_t limit, bool verbose);

/// The sparse class map cross-check of [start_even, limit] (no statistics).
RunStats run_gpu_sparse(uint64_t limit, uint64_t segment_even, const std::string& spv_path,
                        bool verbose, uint64_t start_even, uint32_t split_p,
                        const char* prime_cache_path, bool collect_segments);

} // namespace gb
