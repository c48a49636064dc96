// k_noalloc.cu -- gbc_class_map_noalloc: the tile sieve's class map of a q
// range, built into a buffer the caller owns, with no device allocation.
//
// Some callers cannot call cudaMalloc: code that lives inside another
// framework's memory pool with a fixed device budget (an allocation outside
// the pool is refused or breaks the pool's accounting), and latency-critical
// paths where cudaMalloc's implicit device-wide synchronization is not
// acceptable. The scratch the sieve needs besides its input (the sieving
// primes) and its output (the class map) -- one reciprocal per prime and one
// first class bit per prime and class -- lives in the file-scope device array
// below, which every GPU that loads this library holds until the process
// exits. The pattern words of the primes 7..67 are a constant device table,
// computed at compile time.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "gbc_common.cuh"

namespace {

constexpr uint32_t kTileLog2 = 16;          // 64 Ki bits of a class array per CTA
constexpr uint32_t kFirstTilePrimeIdx = 18; // 71 among the odd primes 3, 5, 7, ...
constexpr uint32_t kWarpPrimeIdx = 171;     // 1031: the first prime >= 2^16 / 64
constexpr size_t kScratchWords = size_t(9) * GBC_NOALLOC_MAX_PRIMES;

// floor(2^32 / p) per prime | 8 first class bits per prime
__device__ __align__(256) static uint32_t g_scratch[kScratchWords];

// ---- the pattern groups of the primes 7..67, at compile time --------------
// canonical bit y of group g's pattern is set iff y mod P_g has no factor
// in the group; the tile kernel shifts each pattern to its tile's phase
constexpr uint32_t kGroupPrimes[gbk::kNumGroups][3] = {{7, 11, 13},  {17, 19, 23}, {29, 31, 1}, {37, 41, 1},
                                                       {43, 47, 1}, {53, 59, 1},   {61, 67, 1}};

constexpr uint32_t group_period(int g) { return kGroupPrimes[g][0] * kGroupPrimes[g][1] * kGroupPrimes[g][2]; }
constexpr uint32_t group_words(int g) { return (group_period(g) + 64 + 31) / 32 + 1; }
constexpr uint32_t pattern_words()
{
    uint32_t t = 0;
    for (int g = 0; g < gbk::kNumGroups; ++g) t += group_words(g);
    return t;
}
constexpr uint32_t kPatWords = pattern_words();  // 653

struct PatternTable {
    uint32_t w[kPatWords];  // first member: the table's address is the words' address
    gbk::GroupInfo gi;
};

constexpr uint32_t inv_mod_small(uint32_t a, uint32_t m)  // a^-1 mod m by search (m < 2^13)
{
    for (uint32_t x = 1; x < m; ++x)
        if (a * x % m == 1) return x;
    return 0;
}

constexpr PatternTable make_pattern_table()
{
    PatternTable t{};
    uint32_t o = 0;
    for (int g = 0; g < gbk::kNumGroups; ++g) {
        const uint32_t P = group_period(g);
        t.gi.P[g] = P;
        t.gi.off[g] = o;
        t.gi.inv30[g] = inv_mod_small(30 % P, P);
        for (uint32_t wd = 0; wd < group_words(g); ++wd) {
            uint32_t v = 0;
            for (uint32_t b = 0; b < 32; ++b) {
                const uint32_t y = (wd * 32 + b) % P;
                bool keep = true;
                for (int j = 0; j < 3; ++j)
                    if (kGroupPrimes[g][j] > 1 && y % kGroupPrimes[g][j] == 0) keep = false;
                if (keep) v |= 1u << b;
            }
            t.w[o + wd] = v;
        }
        o += group_words(g);
    }
    t.gi.words = o;
    return t;
}

constexpr PatternTable kPatterns = make_pattern_table();
__device__ const PatternTable g_patterns = make_pattern_table();

// ---- the host check of the prime list ---------------------------------------
// The kernels take primes[18] = 71 as the first tile-sieve prime, so the list
// must be every odd prime from 3 up to max_prime. A list of nprimes ascending
// odd primes ending at max_prime is that list iff nprimes equals the number
// of odd primes <= max_prime; that count comes from a fixed host table
// (static storage, built once) over every odd number below kCountBound,
// which lies above the GBC_NOALLOC_MAX_PRIMES-th odd prime (1,742,539).
constexpr uint32_t kCountBound = 1u << 21;
constexpr uint32_t kCountWords = kCountBound / 128;  // 64 odd numbers per word
uint64_t g_odd_prime_bits[kCountWords];              // bit j of word w <-> 128 w + 2 j + 1 prime
uint32_t g_odd_prime_pref[kCountWords + 1];          // odd primes in words below w
std::once_flag g_count_once;

void build_prime_count()
{
    for (uint32_t w = 0; w < kCountWords; ++w) g_odd_prime_bits[w] = ~0ull;
    g_odd_prime_bits[0] &= ~1ull;  // 1
    for (uint32_t p = 3; p * p < kCountBound; p += 2) {
        const uint32_t j = p >> 1;
        if (!((g_odd_prime_bits[j >> 6] >> (j & 63)) & 1)) continue;
        for (uint32_t m = p * p; m < kCountBound; m += 2 * p) {
            const uint32_t i = m >> 1;
            g_odd_prime_bits[i >> 6] &= ~(1ull << (i & 63));
        }
    }
    g_odd_prime_pref[0] = 0;
    for (uint32_t w = 0; w < kCountWords; ++w)
        g_odd_prime_pref[w + 1] = g_odd_prime_pref[w] + uint32_t(__builtin_popcountll(g_odd_prime_bits[w]));
}

// odd primes <= x (x < kCountBound)
uint32_t odd_primes_upto(uint32_t x)
{
    std::call_once(g_count_once, build_prime_count);
    const uint32_t n = (x + 1) >> 1;  // odd numbers 1, 3, ..., below x + 1: indices [0, n)
    const uint32_t w = n >> 6, b = n & 63;
    uint32_t c = g_odd_prime_pref[w];
    if (b) c += uint32_t(__builtin_popcountll(g_odd_prime_bits[w] & ((1ull << b) - 1)));
    return c;
}

int set_error(char *err, size_t cap, int code, const char *msg)
{
    if (err && cap) std::snprintf(err, cap, "%s", msg);
    return code;
}

__global__ void k_noalloc_magic(const uint32_t *primes, uint32_t n, uint32_t *magic)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        magic[i] = uint32_t((1ull << 32) / primes[i]);
}

// bits t >= nblk of each class array: cleared, so the map past the range is
// zero (the tile sieve writes whole tiles)
__global__ void k_noalloc_tail(uint32_t *map, uint32_t nblk, uint32_t wpc)
{
    const uint32_t w0 = nblk >> 5, nw = wpc - w0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 8 * nw; i += gridDim.x * blockDim.x) {
        const uint32_t k = i / nw, w = w0 + (i - k * nw);
        uint32_t *a = map + size_t(k) * wpc + w;
        if (w == w0) {
            const uint32_t keep = nblk & 31;
            *a &= keep ? (1u << keep) - 1u : 0u;
        } else {
            *a = 0;
        }
    }
}

}  // namespace

extern "C" int gbc_class_map_noalloc(uint64_t q_lo, uint64_t q_hi, const uint32_t *d_primes, uint32_t nprimes,
                                     uint32_t max_prime, uint32_t *d_map, uint64_t map_words, uint64_t *base_out,
                                     uint32_t *nblk_out, uint32_t *wpc_out, void *stream, char *err, size_t err_cap)
{
    if (q_hi < q_lo || q_hi > GBC_MAX_LIMIT)
        return set_error(err, err_cap, GBC_E_ARG, "need q_lo <= q_hi <= 2^64 - 2^40");
    if (q_hi - q_lo > GBC_NOALLOC_MAX_SPAN)
        return set_error(err, err_cap, GBC_E_ARG, "q range wider than GBC_NOALLOC_MAX_SPAN (2^30)");
    if (!d_primes || !nprimes || nprimes > GBC_NOALLOC_MAX_PRIMES)
        return set_error(err, err_cap, GBC_E_ARG, "nprimes must be in [1, GBC_NOALLOC_MAX_PRIMES = 131072]");
    if (max_prime >= kCountBound || odd_primes_upto(max_prime) != nprimes)
        return set_error(err, err_cap, GBC_E_ARG,
                         "d_primes must hold every odd prime from 3 to max_prime (nprimes differs from their count)");
    const uint64_t pb = max_prime < 67 ? 67 : max_prime;
    if (pb * pb < q_hi)
        return set_error(err, err_cap, GBC_E_ARG, "the primes end below sqrt(q_hi): the map would not be exact");

    const uint32_t tb = 1u << kTileLog2, tw = tb / 32;
    gbk::BatchParams bp{};
    bp.base = q_lo / 30 * 30;
    bp.qmax = q_hi;
    const uint64_t nblk = (q_hi - bp.base) / 30 + 1;
    const uint64_t tiles = (nblk + 64 + tb - 1) / tb;
    bp.nblk = uint32_t(nblk);
    bp.tiles_pc = uint32_t(tiles);
    bp.tb_tiles = bp.tiles_pc;
    bp.wpc = uint32_t(tiles * tw);
    if (base_out) *base_out = bp.base;
    if (nblk_out) *nblk_out = bp.nblk;
    if (wpc_out) *wpc_out = bp.wpc;
    if (!d_map || map_words < uint64_t(8) * bp.wpc)
        return set_error(err, err_cap, GBC_E_ARG, "map buffer smaller than 8 * wpc words (wpc is returned)");

    // the device addresses of the scratch array and the pattern table on the
    // current device, looked up on every call (no cached address can outlive
    // a reset of the device's context)
    void *scratch_v = nullptr, *pat_v = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&scratch_v, g_scratch);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&pat_v, g_patterns);
    if (e != cudaSuccess) return set_error(err, err_cap, GBC_E_CUDA, cudaGetErrorString(e));
    uint32_t *scratch = static_cast<uint32_t *>(scratch_v);
    bp.map = d_map;
    bp.primes = d_primes;
    bp.pat = static_cast<const uint32_t *>(pat_v);
    bp.magic = scratch;
    bp.xfirst = scratch + GBC_NOALLOC_MAX_PRIMES;
    bp.tile_log2 = kTileLog2;
    bp.i0 = nprimes < kFirstTilePrimeIdx ? nprimes : kFirstTilePrimeIdx;
    bp.n_mid = nprimes;
    bp.n_all = nprimes;
    bp.i_warp = nprimes < kWarpPrimeIdx ? nprimes : kWarpPrimeIdx;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // every scratch word a kernel reads is written earlier in this call:
    // nothing needs clearing
    k_noalloc_magic<<<64, 256, 0, st>>>(d_primes, nprimes, scratch);
    gbh::launch_xfirst1(bp, st);
    gbh::launch_tile1(bp, kPatterns.gi, st);  // 2^16-bit tiles: under the default shared-memory limit
    const uint32_t tail_words = 8 * (bp.wpc - (bp.nblk >> 5));
    k_noalloc_tail<<<(tail_words + 255) / 256, 256, 0, st>>>(d_map, bp.nblk, bp.wpc);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(err, err_cap, GBC_E_CUDA, cudaGetErrorString(e));
    return GBC_OK;
}
