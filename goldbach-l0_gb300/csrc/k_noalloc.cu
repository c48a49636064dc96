// k_noalloc.cu -- gbc_class_map_noalloc: the tile sieve's class map of a q
// range, built into a buffer the caller owns, with no device allocation.
//
// Callers that cannot call cudaMalloc use this entry point: code that runs
// while a CUDA stream is being captured, code that lives inside another
// framework's memory pool with a fixed device budget, and latency-critical
// paths where cudaMalloc's implicit device-wide synchronization is not
// acceptable. The scratch the sieve needs besides its input (the sieving
// primes) and its output (the class map) -- the pattern words of the primes
// 7..67, one reciprocal per prime and one first class bit per prime and
// class -- lives in the file-scope device array below, which every GPU that
// loads this library holds until the process exits.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <vector>

#include "gbc_common.cuh"

namespace {

constexpr uint32_t kTileLog2 = 16;          // 64 Ki bits of a class array per CTA
constexpr uint32_t kPatWords = 1024;        // room for the seven group patterns (640 words)
constexpr uint32_t kFirstTilePrimeIdx = 18; // 71 among the odd primes 3, 5, 7, ...
constexpr uint32_t kWarpPrimeIdx = 171;     // 1031: the first prime >= 2^16 / 64
constexpr size_t kScratchWords = kPatWords + size_t(9) * GBC_NOALLOC_MAX_PRIMES;

// pattern words | floor(2^32 / p) per prime | 8 first class bits per prime
__device__ __align__(256) static uint32_t g_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
uint32_t *g_scratch_ptr[kMaxDevices];  // device address of g_scratch, per device
gbk::GroupInfo g_groups;
std::mutex g_mu;

constexpr uint32_t kGroupPrimes[gbk::kNumGroups][3] = {{7, 11, 13},  {17, 19, 23}, {29, 31, 1}, {37, 41, 1},
                                                       {43, 47, 1}, {53, 59, 1},   {61, 67, 1}};

uint32_t inv_mod(uint32_t a, uint32_t m)
{
    for (uint32_t x = 1; x < m; ++x)
        if (uint64_t(a) * x % m == 1) return x;
    return 0;
}

// The canonical group patterns (bit y set iff y mod P has no factor in the
// group) and their descriptors, the tables gbc_create builds.
std::vector<uint32_t> make_patterns(gbk::GroupInfo &gi)
{
    std::vector<uint32_t> pat;
    for (int g = 0; g < gbk::kNumGroups; ++g) {
        uint32_t P = 1;
        for (int j = 0; j < 3; ++j) P *= kGroupPrimes[g][j];
        const uint32_t words = (P + 64 + 31) / 32 + 1;
        gi.P[g] = P;
        gi.off[g] = uint32_t(pat.size());
        gi.inv30[g] = inv_mod(30 % P, P);
        for (uint32_t w = 0; w < words; ++w) {
            uint32_t v = 0;
            for (uint32_t b = 0; b < 32; ++b) {
                const uint32_t y = (w * 32 + b) % P;
                bool keep = true;
                for (int j = 0; j < 3; ++j)
                    if (kGroupPrimes[g][j] > 1 && y % kGroupPrimes[g][j] == 0) keep = false;
                if (keep) v |= 1u << b;
            }
            pat.push_back(v);
        }
    }
    gi.words = uint32_t(pat.size());
    return pat;
}

int set_error(char *err, size_t cap, int code, const char *msg)
{
    if (err && cap) std::snprintf(err, cap, "%s", msg);
    return code;
}

// Once per device, with the device current: the scratch array's device
// address and the constant pattern words in it.
int setup_device(int dev, char *err, size_t cap)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_scratch_ptr[dev]) return GBC_OK;
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess) return set_error(err, cap, GBC_E_CUDA, cudaGetErrorString(e));
    gbk::GroupInfo gi{};
    const std::vector<uint32_t> pat = make_patterns(gi);
    if (pat.size() > kPatWords) return set_error(err, cap, GBC_E_ARG, "pattern words exceed the scratch slot");
    const cudaError_t e2 = cudaMemcpy(ptr, pat.data(), pat.size() * 4, cudaMemcpyHostToDevice);
    if (e2 != cudaSuccess) return set_error(err, cap, GBC_E_CUDA, cudaGetErrorString(e2));
    g_groups = gi;
    g_scratch_ptr[dev] = static_cast<uint32_t *>(ptr);
    return GBC_OK;
}

__global__ void k_noalloc_magic(const uint32_t *primes, uint32_t n, uint32_t *magic)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        magic[i] = uint32_t((1ull << 32) / primes[i]);
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
    const uint64_t pb = max_prime < 67 ? 67 : max_prime;
    if (pb * pb < q_hi)
        return set_error(err, err_cap, GBC_E_ARG, "the primes end below sqrt(q_hi): the map would not be exact");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(err, err_cap, GBC_E_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(err, err_cap, GBC_E_ARG, "device ordinal above 63");
    if (int rc = setup_device(dev, err, err_cap)) return rc;

    const uint32_t tb = 1u << kTileLog2, tw = tb / 32;
    gbk::BatchParams bp{};
    bp.base = q_lo / 30 * 30;
    bp.qmax = q_hi;
    const uint64_t nblk = (q_hi - bp.base) / 30 + 1;
    const uint64_t tiles = (nblk + 64 + tb - 1) / tb;
    bp.nblk = uint32_t(nblk);
    bp.tiles_pc = uint32_t(tiles);
    bp.wpc = uint32_t(tiles * tw);
    if (base_out) *base_out = bp.base;
    if (nblk_out) *nblk_out = bp.nblk;
    if (wpc_out) *wpc_out = bp.wpc;
    if (!d_map || map_words < uint64_t(8) * bp.wpc)
        return set_error(err, err_cap, GBC_E_ARG, "map buffer smaller than 8 * wpc words (wpc is returned)");
    uint32_t *scratch = g_scratch_ptr[dev];
    bp.map = d_map;
    bp.primes = d_primes;
    bp.pat = scratch;
    bp.magic = scratch + kPatWords;
    bp.xfirst = scratch + kPatWords + GBC_NOALLOC_MAX_PRIMES;
    bp.tile_log2 = kTileLog2;
    bp.i0 = nprimes < kFirstTilePrimeIdx ? nprimes : kFirstTilePrimeIdx;
    bp.n_mid = nprimes;
    bp.n_all = nprimes;
    bp.i_warp = nprimes < kWarpPrimeIdx ? nprimes : kWarpPrimeIdx;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // every scratch word a kernel reads is written earlier in this call:
    // nothing needs clearing
    k_noalloc_magic<<<64, 256, 0, st>>>(d_primes, nprimes, scratch + kPatWords);
    gbh::launch_xfirst1(bp, st);
    gbh::launch_tile1(bp, g_groups, st);  // 2^16-bit tiles: under the default shared-memory limit
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(err, err_cap, GBC_E_CUDA, cudaGetErrorString(e));
    return GBC_OK;
}
