// gb_verifier.cpp -- the reference's C++ entry points (include/gb_verifier.hpp)
// on this library: gb::run_gpu, gb::print_device_info, gb::verify_cpu and
// gb::run_gpu_sparse with the reference's signatures and structs, so the
// reference's callers (src/main.cpp:356-361) link against libgbc.so in place
// of src/verifier.cpp and src/sparse.cpp.
//
// gb::run_gpu (include/verifier.hpp:71-110) here:
//   - spv_path and prime_cache_path are accepted and not used (the kernels
//     are compiled into this library; the sieving primes are computed in
//     memory by every context);
//   - segment_even: the integer span of a segment (0: 467.5M), used as given;
//   - sieve_split_arg: the index of the first odd prime above the tile sieve
//     (the reference's split index); 0 keeps the tuned split (primes up to
//     2^21 in the shared-memory tiles);
//   - the knobs the reference reads from its environment are read the same
//     way, strictly (a malformed value throws before any GPU work): GB_STATS
//     (0/1, default 1: campaign statistics for runs that start at >= 1e6),
//     GB_STATS_SAMPLE (every k-th segment of a run gets p(n) of every even,
//     default 256), GB_GAPS (exact, 1, sampled or 0; every segment's gaps are
//     walked here, so "sampled" records the same exact gaps as "exact"),
//     GB_STATS_STATE / GB_STATS_LOG (goldbach_stats.state / .log), the ridge
//     store, records file, live snapshot and hook (GB_RIDGE, GB_RIDGE_FILE,
//     GB_RECORDS_FILE, GB_STATS_LIVE, GB_RECORD_HOOK) and GB_RIDGE_MIN;
//   - the batched form's tuned knobs (segments per batch up to 128, tiles
//     of 1,835,008 bits, the tile sieve to 1,703,936 and hit lists above it
//     through a multiplier table of up to 160 GB, 16 funnels of which 3 on
//     every word) are this implementation's defaults;
//   - it throws std::runtime_error on any failure, as the reference, and the
//     statistics files are written only after the run passed.
#include "../../include/gb_verifier.hpp"

#include <cuda_runtime_api.h>

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "gb_run.hpp"

namespace gb {

namespace {

// ---- the GB_* environment, parsed strictly (unset or "" = the default) ------

[[noreturn]] void bad_env(const char *name, const char *value, const std::string &accepts)
{
    throw std::runtime_error(std::string(name) + "='" + value + "': expected " + accepts);
}

bool env_onoff(const char *name, bool dflt)
{
    const char *e = std::getenv(name);
    if (!e || !*e) return dflt;
    if (!std::strcmp(e, "0")) return false;
    if (!std::strcmp(e, "1")) return true;
    bad_env(name, e, "0 or 1");
}

uint32_t env_u32(const char *name, uint32_t dflt, uint32_t lo, uint32_t hi)
{
    const char *e = std::getenv(name);
    if (!e) return dflt;
    char *end = nullptr;
    errno = 0;
    const unsigned long long v = (*e >= '0' && *e <= '9') ? std::strtoull(e, &end, 0) : 0;
    if (!(*e >= '0' && *e <= '9') || errno || !end || *end || v < lo || v > hi)
        bad_env(name, e, "an integer in [" + std::to_string(lo) + ", " + std::to_string(hi) + "]");
    return uint32_t(v);
}

std::string env_choice(const char *name, const char *dflt, std::initializer_list<const char *> allowed)
{
    const char *e = std::getenv(name);
    if (!e || !*e) return dflt;
    for (const char *a : allowed)
        if (!std::strcmp(e, a)) return e;
    std::string acc;
    for (const char *a : allowed) acc += (acc.empty() ? "" : ", ") + std::string(a);
    bad_env(name, e, "one of " + acc);
}

std::string env_path(const char *name, const char *dflt)
{
    const char *e = std::getenv(name);
    return e && *e ? e : dflt;
}

// odd primes up to n (the host's view of the sieving primes, for the split index)
std::vector<uint32_t> odd_primes_upto(uint32_t n)
{
    std::vector<uint8_t> c(n / 2 + 1, 1);
    std::vector<uint32_t> out;
    for (uint32_t i = 1; 2 * i + 1 <= n; ++i) {
        if (!c[i]) continue;
        const uint64_t p = 2 * i + 1;
        out.push_back(uint32_t(p));
        for (uint64_t m = p * p; m <= n; m += 2 * p) c[m / 2] = 0;
    }
    return out;
}

struct CtxCloser {
    void operator()(gbc_ctx *c) const { gbc_destroy(c); }
};

double since(std::chrono::steady_clock::time_point t)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}

constexpr uint32_t kTileBits = 1835008;     // bits per shared-memory tile (224 KB)
constexpr uint32_t kTunedPmid = 1703936;    // primes to 1.625 * 2^20 in the shared-memory tiles (the tuned split)
constexpr uint32_t kMaskPrimes = 16;        // 7..67 by whole-word patterns

}  // namespace

RunStats run_gpu(uint64_t limit, uint64_t segment_even, const std::string &spv_path, bool verbose, uint64_t start_even,
                 uint32_t sieve_split_arg, const char *prime_cache_path, bool collect_segments)
{
    (void)spv_path;
    (void)prime_cache_path;
    const auto t0 = std::chrono::steady_clock::now();
    uint64_t start = std::max<uint64_t>(start_even, 4);
    start += start & 1;
    limit &= ~uint64_t(1);
    if (limit < 4 || limit > GBC_MAX_LIMIT)
        throw std::runtime_error("limit " + std::to_string(limit) + " outside [4, 2^64 - 2^40]");
    if (start > limit) throw std::runtime_error("no even n in [start, limit]");
    const uint64_t seg = segment_even ? (segment_even + 1) & ~uint64_t(1) : GBC_DEFAULT_SEGMENT;
    // the knobs, read up front (a malformed one fails before any GPU work)
    const bool stats_on = start >= kStatsMinStart && env_onoff("GB_STATS", true);
    const std::string gaps = env_choice("GB_GAPS", "exact", {"exact", "1", "sampled", "0"});
    const uint32_t sample = env_u32("GB_STATS_SAMPLE", 256, 1, UINT32_MAX - 1);  // segment 0 always sampled
    const uint32_t ridge_min = env_u32("GB_RIDGE_MIN", GBC_TAIL_T, 0, UINT32_MAX);
    uint32_t p_mid = kTunedPmid, split_used = 0;
    {
        const std::vector<uint32_t> small = odd_primes_upto(1u << 23);
        if (sieve_split_arg) {
            if (sieve_split_arg >= small.size() || small[sieve_split_arg] < 1024)
                throw std::runtime_error("sieve split index " + std::to_string(sieve_split_arg) +
                                         " outside this implementation's tile range (primes 1024 .. 2^23)");
            p_mid = small[sieve_split_arg - 1];
        }
        split_used = uint32_t(std::upper_bound(small.begin(), small.end(), p_mid) - small.begin());
    }
    const auto segs = plan_segments(start, limit, seg);
    gbc_config cfg{};
    cfg.limit = limit;
    cfg.segment_even = seg;
    cfg.max_batch = uint32_t(std::min<size_t>(128, segs.size()));
    cfg.p_mid = p_mid;
    cfg.mtab_max_gb = 160;
    cfg.tile_log2 = 20;
    cfg.tile_bits = kTileBits;
    cfg.plan_funnels = 16;
    cfg.verify_funnels = 3;
    cfg.sample_every = sample;
    cfg.ridge_min = std::max<uint32_t>(ridge_min, GBC_TAIL_T);  // the plan's phase-A ceiling (ridge.hpp:89)
    gbc_ctx *raw = nullptr;
    const int rc = gbc_create(&cfg, &raw);
    std::unique_ptr<gbc_ctx, CtxCloser> ctx(raw);
    if (rc != GBC_OK) throw GbcError(rc, std::string("gbc_create: ") + gbc_last_error(raw));
    const double create_s = since(t0);
    attach_env_outputs(ctx.get());
    if (stats_on) {
        const std::string state = env_path("GB_STATS_STATE", "goldbach_stats.state");
        const std::string log = env_path("GB_STATS_LOG", "goldbach_stats.log");
        if (int r = gbc_set_stats(ctx.get(), state.c_str(), log.c_str(), kVersion, gaps != "0"))
            throw GbcError(r, gbc_last_error(ctx.get()));
    }
    const auto t1 = std::chrono::steady_clock::now();
    if (int r = gbc_prepare(ctx.get(), start, limit)) throw GbcError(r, std::string("prepare: ") + gbc_last_error(ctx.get()));
    const double upload_s = since(t1);
    const RangeStats rs = run_range(ctx.get(), start, limit, seg, cfg.max_batch, nullptr, nullptr,
                                    stats_on ? sample : 256, collect_segments);

    RunStats st;
    st.limit = limit;
    st.start = start;
    st.segments = rs.segments;
    st.leftovers = rs.leftovers;
    st.init_cache_s = create_s;
    st.init_upload_s = upload_s;
    st.init_seconds = create_s + upload_s;
    st.gpu_seconds = rs.wall_seconds;
    st.total_seconds = st.init_seconds + st.gpu_seconds;
    st.evens_per_second = rs.wall_seconds > 0 ? double(rs.evens) / rs.wall_seconds : 0.0;
    st.sieve_seconds = rs.tile_ms / 1e3;
    st.large_seconds = rs.large_ms / 1e3;
    st.verify_seconds = (rs.check_ms + rs.count_ms) / 1e3;
    st.sync_seconds = std::max(0.0, st.gpu_seconds - st.sieve_seconds - st.large_seconds - st.verify_seconds);
    st.split_used = split_used;
    for (const auto &s : segs) {
        const uint64_t bits = (s.second - s.first + GBC_MAX_CAND + 30) / 30 + 1;
        st.total_tiles += 8 * ((bits + kTileBits - 1) / kTileBits);
    }
    if (const Outputs *o = outputs_of(ctx.get())) {
        st.ridge_min = cfg.ridge_min;
        st.ridge_found = o->ridges().appends();
        st.ridge_dropped = o->ridges().dropped();
        for (const RidgeRow &r : o->ridges().top()) st.ridge_top.push_back({r.n, r.p, r.q, r.seg, r.found});
    }
    if (stats_on) {
        st.stats_on = true;
        st.stats_pmax = rs.pmax;
        st.stats_primes = rs.primes;
        st.stats_twins = rs.twins;
        st.stats_sampled = rs.evens_sampled;
        st.stats_tail = rs.tail_evens;
    }
    if (collect_segments)
        for (const SegRecord &r : rs.per_segment) {
            SegmentStats s;
            s.seg_start = r.start;
            s.seg_end = r.end;
            s.evens = r.evens;
            const uint64_t bits = (r.end - r.start + GBC_MAX_CAND + 30) / 30 + 1;
            s.tiles = 8 * ((bits + kTileBits - 1) / kTileBits);
            s.sieve_split = split_used;
            s.mask_count = kMaskPrimes;
            s.leftovers = r.leftovers;
            s.sieve_seconds = r.tile_ms / 1e3;
            s.large_seconds = r.large_ms / 1e3;
            s.check_seconds = r.check_ms / 1e3;
            s.wall_seconds = r.wall_ms / 1e3;
            st.per_segment.push_back(s);
        }
    if (verbose)
        std::printf("run [%" PRIu64 ", %" PRIu64 "]: %" PRIu64 " segments in %" PRIu64 " batches, init %.3f s, "
                    "loop %.3f s (sieve %.3f, large %.3f, check %.3f s device), %.3f G evens/s\n",
                    st.start, st.limit, st.segments, rs.batches, st.init_seconds, st.gpu_seconds, st.sieve_seconds,
                    st.large_seconds, st.verify_seconds, st.evens_per_second / 1e9);
    return st;
}

void print_device_info()
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) throw std::runtime_error("no CUDA GPU is reported");
    int drv = 0, rtv = 0;
    cudaDriverGetVersion(&drv);
    cudaRuntimeGetVersion(&rtv);
    for (int d = 0; d < n; ++d) {
        cudaDeviceProp p{};
        if (cudaGetDeviceProperties(&p, d) != cudaSuccess) throw std::runtime_error("cudaGetDeviceProperties failed");
        int sm_clock = 0, mem_clock = 0, bus = 0, l2 = 0, smem = 0;
        cudaDeviceGetAttribute(&sm_clock, cudaDevAttrClockRate, d);
        cudaDeviceGetAttribute(&mem_clock, cudaDevAttrMemoryClockRate, d);
        cudaDeviceGetAttribute(&bus, cudaDevAttrGlobalMemoryBusWidth, d);
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, d);
        cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, d);
        std::printf("device           : %d %s (compute capability %d.%d)\n", d, p.name, p.major, p.minor);
        std::printf("multiprocessors  : %d (max threads per SM %d)\n", p.multiProcessorCount,
                    p.maxThreadsPerMultiProcessor);
        std::printf("SM clock         : %d MHz\n", sm_clock / 1000);
        std::printf("memory           : %.1f GB (%d MHz, %d-bit), L2 %.1f MB\n", double(p.totalGlobalMem) / double(1ull << 30),
                    mem_clock / 1000, bus, double(l2) / double(1 << 20));
        std::printf("shared memory    : %d KB per block (opt-in)\n", smem / 1024);
        std::printf("driver / runtime : %d / %d\n", drv, rtv);
    }
    std::printf("build            : segment %llu integers, tile %u bits, tile primes <= %u, hit lists through the "
                "prime-multiplier table, candidates 3..%u, statistics tail %u, version %s\n",
                (unsigned long long)GBC_DEFAULT_SEGMENT, kTileBits, kTunedPmid, GBC_MAX_CAND, GBC_TAIL_T, kVersion);
}

bool verify_cpu(uint64_t limit, bool verbose)
{
    const auto prime = [](uint64_t n) {
        if (n < 2) return false;
        if (n % 2 == 0) return n == 2;
        for (uint64_t d = 3; d * d <= n; d += 2)
            if (n % d == 0) return false;
        return true;
    };
    for (uint64_t n = 4; n <= limit; n += 2) {
        bool ok = false;
        for (uint64_t p = 2; p <= n / 2 && !ok; p = p == 2 ? 3 : p + 2) ok = prime(p) && prime(n - p);
        if (!ok) {
            if (verbose) std::printf("no Goldbach partition for n = %llu\n", (unsigned long long)n);
            return false;
        }
        if (verbose && n % 1000000 == 0) std::printf("cpu check: %llu\n", (unsigned long long)n);
    }
    return true;
}

RunStats run_gpu_sparse(uint64_t limit, uint64_t segment_even, const std::string &spv_path, bool verbose,
                        uint64_t start_even, uint32_t split_p, const char *prime_cache_path, bool collect_segments)
{
    (void)spv_path;
    (void)prime_cache_path;
    (void)split_p;           // the sparse sieve's tile / large split is fixed at 2^20 here
    (void)collect_segments;  // no per-segment records on the sparse path
    constexpr uint64_t kM = 30030;
    uint32_t dlt_log2 = 0;   // the default 2^26 evens per class and segment
    if (segment_even && segment_even != GBC_DEFAULT_SEGMENT) {
        const uint64_t dlt = std::max<uint64_t>(segment_even / kM, 4096);
        dlt_log2 = std::min<uint32_t>(26, std::max<uint32_t>(12, uint32_t(std::floor(std::log2(double(dlt))))));
    }
    const auto t0 = std::chrono::steady_clock::now();
    const RangeStats rs = run_sparse(limit, verbose, start_even, dlt_log2);
    RunStats st;
    st.limit = rs.limit;
    st.start = rs.start;
    st.segment_used = kM << (dlt_log2 ? dlt_log2 : 26);
    st.segments = rs.segments;
    st.leftovers = rs.leftovers;
    st.gpu_seconds = rs.wall_seconds;
    st.total_seconds = since(t0);
    st.init_seconds = std::max(0.0, st.total_seconds - st.gpu_seconds);
    st.evens_per_second = rs.wall_seconds > 0 ? double(rs.evens) / rs.wall_seconds : 0.0;
    st.sieve_seconds = rs.tile_ms / 1e3;
    st.large_seconds = rs.large_ms / 1e3;
    st.verify_seconds = rs.check_ms / 1e3;
    st.sync_seconds = std::max(0.0, st.gpu_seconds - st.sieve_seconds - st.large_seconds - st.verify_seconds);
    return st;
}

}  // namespace gb
