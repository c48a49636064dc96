// k_sparse.cu -- the sparse class map: an independent, verify-only
// cross-check of Goldbach's conjecture on a range (the reference's opt-in
// `--sparse` path: include/sparse.hpp, src/sparse.cpp, kernels/sparse.cl),
// designed here for one GB300.
//
// Every even n needs one certified prime q = n - p. The map holds only the
// q of K = 12 residue classes c_k mod M = 30030; every even class r = n mod M
// reaches at least one class k with r - c_k a unit (the residues below are
// built so), and the candidates p = ((r - c_k) mod M) + M a <= pmax of those
// classes test the map bits t = i + U, U = TB - a - [r < c_k], of the evens
// n = N + r + M i: one 64-bit funnel shift per 32 evens and candidate.
//
// Per segment (evens [N, N + M dl), map bits t < T = dl + TB of K rows):
//   k_sp_first  per sieving prime below 2^20 and class: the first bit t of a
//               multiple (q = p m with m = c_k p^-1 mod M, from an inverse
//               table mod M: no inverse mod p is ever computed)
//   k_sp_tile   persistent CTAs over (class, 2^20-bit tile) items: the tile
//               in shared memory, primes below 2^10 warp-cooperatively, the
//               rest a thread per prime, one coalesced store (bits >= T zero)
//   k_sp_large  a thread per prime from 2^20: its twelve first bits, each mark
//               a read of the word and an atomic AND only where the bit is set
//   k_sp_popc   set bits of the map
//   k_sp_check  persistent CTAs over (chunk of 4096 evens per class, block of
//               1024 even classes) items; each item's twelve row windows are
//               staged in shared memory by bulk copies (two buffers: the next
//               item's copies land while this one is checked); a warp takes an
//               even class, each lane four words of its evens, and ORs in the
//               plan entries (class, window word, up to six packed offsets) in
//               plan order until every even of the warp is verified; words left
//               unverified go to the pending list, which the host resolves by
//               an ascending Miller-Rabin scan.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gbc.h"
#include "gbc_common.cuh"
#include "gbc_internal.h"

namespace gbs {

constexpr uint32_t kM = 30030, kHalfM = 15015, kK = 12;
constexpr uint32_t kTileLog2 = 20, kTileBits = 1u << kTileLog2, kTileWords = kTileBits / 32;
constexpr uint32_t kSplit = 1u << 20;        // sieving primes below: tiles; from: k_sp_large
constexpr uint32_t kWarpPrime = 1024;        // below: a warp per prime in the tile
constexpr uint32_t kV = 4;                   // words per lane in the checker
constexpr uint32_t kChunkWords = 32 * kV;    // words (of evens) per class and checker item
constexpr uint32_t kChunkEvens = 32 * kChunkWords;
constexpr uint32_t kCheckWarps = 8, kCheckThreads = 32 * kCheckWarps;
constexpr uint32_t kClassBlock = 128 * kCheckWarps;  // even classes per checker item
constexpr uint32_t kClassBlocks = (kHalfM + kClassBlock - 1) / kClassBlock;
constexpr uint32_t kPendCap = 1u << 20;      // pending words per segment
constexpr uint32_t kErrStaging = 1u << 0;    // a bulk copy missed its wait limit
constexpr uint32_t kEntryMax = 6;            // candidates per plan entry

// A plan entry: up to six candidates of one class k and one window word o,
// as x = k | o << 4 | count << 12 and y = their offsets within the word, 5
// bits each, ascending (an odd count repeats the last offset, so entries
// are taken two offsets at a time; a funnel shift reads only an offset's
// low five bits, so y >> 5 j needs no mask).
__host__ __device__ __forceinline__ uint32_t entry_k(uint32_t x) { return x & 15u; }
__host__ __device__ __forceinline__ uint32_t entry_o(uint32_t x) { return (x >> 4) & 255u; }
__host__ __device__ __forceinline__ uint32_t entry_n(uint32_t x) { return (x >> 12) & 7u; }

// inverse of a odd mod 2^64 (Newton: each step doubles the correct bits)
constexpr uint64_t inv64(uint64_t a)
{
    uint64_t x = a;
    for (int i = 0; i < 6; ++i) x *= 2 - a * x;
    return x;
}
constexpr uint64_t kInvHalfM = inv64(kHalfM);
static_assert(kInvHalfM * kHalfM == 1, "inverse of M / 2 mod 2^64");

struct SpCtr {
    unsigned long long map_primes, groups, evens;
    uint32_t npend, err, work_tile, work_check;
};

// one segment, by value to every kernel
struct SpSeg {
    uint64_t N, Q;            // first even; q of bit 0 minus c_k (N - M TB)
    uint64_t start, limit;    // the evens verified: [start, limit] within the segment
    uint32_t dl, T, tb;       // evens per class; map bits per row (dl + TB); TB
    uint32_t tiles, chunks;   // tiles per row; checker chunks
    uint32_t stride, rw;      // words per map row; staged words per row and item
    uint32_t group_cap;       // plan entries per class (all: ~0)
    uint32_t *map;
    SpCtr *ctr;
    uint32_t c[kK];           // residues
};

// First bit t of a multiple of p in each class row: q = p m, m = c_k p^-1
// (mod M), the least such m with p m >= Q; then (p m - Q - c_k) / M, an
// exact division (by 2, then by the inverse of M / 2 mod 2^64). t < p:
// p m - Q < p M, since the m one period lower gives a multiple below Q.
__device__ __forceinline__ void sp_first(uint64_t Q, uint32_t p, uint32_t invp, const uint32_t *c, uint64_t *t)
{
    const uint64_t qd = Q / p;
    const uint64_t mlo = qd + (Q - qd * p != 0 ? 1 : 0);
    const uint32_t mm = uint32_t(mlo % kM);
#pragma unroll
    for (uint32_t k = 0; k < kK; ++k) {
        const uint32_t mu = (c[k] * invp) % kM;
        const uint32_t d = mu >= mm ? mu - mm : mu + kM - mm;
        const uint64_t q = uint64_t(p) * (mlo + d);
        t[k] = ((q - Q - c[k]) >> 1) * kInvHalfM;
    }
}

__global__ void __launch_bounds__(256) k_sp_first(SpSeg s, const uint32_t *primes, uint32_t nsmall,
                                                  const uint16_t *inv, uint32_t *xf)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nsmall; i += gridDim.x * blockDim.x) {
        const uint32_t p = primes[i];
        uint64_t t[kK];
        sp_first(s.Q, p, inv[p % kM], s.c, t);
#pragma unroll
        for (uint32_t k = 0; k < kK; ++k) xf[size_t(k) * nsmall + i] = uint32_t(t[k]);
    }
}

// first multiple at or after tile start ts from the row's first bit t0
__device__ __forceinline__ uint32_t tile_first(uint32_t t0, uint32_t ts, uint32_t p)
{
    if (t0 >= ts) return t0 - ts;
    const uint32_t r = (ts - t0) % p;
    return r ? p - r : 0;
}

__global__ void __launch_bounds__(1024, 1) k_sp_tile(SpSeg s, const uint32_t *primes, uint32_t nsmall,
                                                     uint32_t nwarp, const uint32_t *xf)
{
    extern __shared__ __align__(16) uint32_t tw[];
    __shared__ uint32_t s_j;
    const uint32_t tid = threadIdx.x, bs = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = bs >> 5;
    const uint32_t items = kK * s.tiles;
    for (;;) {
        const uint32_t j = gbk::next_item(&s.ctr->work_tile, &s_j);
        if (j >= items) break;
        const uint32_t k = j / s.tiles, ts = (j - k * s.tiles) << kTileLog2;
        for (uint32_t w = tid; w < kTileWords; w += bs) tw[w] = ~0u;
        __syncthreads();
        const uint32_t *xk = xf + size_t(k) * nsmall;
        for (uint32_t i = warp; i < nwarp; i += nw) {
            const uint32_t p = __ldg(primes + i);
            const uint32_t l = tile_first(__ldg(xk + i), ts, p);
            for (uint32_t b = l + lane * p; b < kTileBits; b += 32 * p) atomicAnd(&tw[b >> 5], ~(1u << (b & 31)));
        }
        for (uint32_t i = nwarp + tid; i < nsmall; i += bs) {
            const uint32_t p = __ldg(primes + i);
            const uint32_t l = tile_first(__ldg(xk + i), ts, p);
            for (uint32_t b = l; b < kTileBits; b += p) atomicAnd(&tw[b >> 5], ~(1u << (b & 31)));
        }
        __syncthreads();
        uint32_t *dst = s.map + size_t(k) * s.stride + (ts >> 5);
        for (uint32_t w = tid; w < kTileWords; w += bs) {
            const uint32_t t0 = ts + 32 * w;
            uint32_t v = tw[w];
            if (t0 + 32 > s.T) v = t0 >= s.T ? 0u : v & ((1u << (s.T - t0)) - 1u);
            dst[w] = v;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_sp_large(SpSeg s, const uint32_t *primes, uint32_t i0, uint32_t n,
                                                  const uint16_t *inv)
{
    for (uint32_t i = i0 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = __ldg(primes + i);
        uint64_t t[kK];
        sp_first(s.Q, p, __ldg(inv + p % kM), s.c, t);
#pragma unroll
        for (uint32_t k = 0; k < kK; ++k) {
            uint32_t *row = s.map + size_t(k) * s.stride;
            for (uint64_t x = t[k]; x < s.T; x += p) {
                uint32_t *w = row + (x >> 5);
                const uint32_t bit = 1u << (x & 31);
                if (__ldcg(w) & bit) atomicAnd(w, ~bit);
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_sp_popc(SpSeg s)
{
    const uint32_t rwords = (s.T + 31) / 32;
    const uint64_t total = uint64_t(kK) * rwords;
    unsigned long long sum = 0;
    for (uint64_t x = blockIdx.x * blockDim.x + threadIdx.x; x < total; x += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t k = uint32_t(x / rwords), w = uint32_t(x - uint64_t(k) * rwords);
        sum += __popc(s.map[size_t(k) * s.stride + w]);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) sum += __shfl_down_sync(~0u, sum, o);
    if ((threadIdx.x & 31) == 0 && sum) atomicAdd(&s.ctr->map_primes, sum);
}

// bits [0, x) of a word, x <= 32
__device__ __forceinline__ uint32_t low_bits(uint32_t x) { return x >= 32 ? ~0u : (1u << x) - 1u; }

// the twelve row windows of chunk c into buf: row k's words [c W, c W + rw)
__device__ __forceinline__ void sp_stage(const SpSeg &s, uint32_t *buf, uint64_t *bar, uint32_t c)
{
    gbk::fence_proxy_async();
    gbk::mbar_arrive_expect_tx(bar, kK * s.rw * 4);
#pragma unroll 1
    for (uint32_t k = 0; k < kK; ++k)
        gbk::bulk_copy_g2s(buf + k * s.rw, s.map + size_t(k) * s.stride + size_t(c) * kChunkWords, s.rw * 4, bar);
}

__global__ void __launch_bounds__(kCheckThreads, 4) k_sp_check(SpSeg s, const uint2 *groups, const uint32_t *goff,
                                                            uint4 *pend)
{
    extern __shared__ __align__(16) uint32_t win[];  // two buffers of kK * rw words
    __shared__ uint64_t s_bar[2];
    __shared__ uint32_t s_j[2];  // alternate: no barrier separates two item fetches
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t items = s.chunks * kClassBlocks;
    if (tid == 0) {
        gbk::mbar_init(&s_bar[0], 1);
        gbk::mbar_init(&s_bar[1], 1);
        gbk::mbar_init_fence();
    }
    uint32_t phase = 0, buf = 0;
    unsigned long long ngroups = 0, nevens = 0;
    uint32_t j = gbk::next_item(&s.ctr->work_check, &s_j[0]);
    if (j < items && tid == 0) sp_stage(s, win, &s_bar[0], j / kClassBlocks);
    while (j < items) {
        // the next item's copies go into the other buffer, free since the
        // synchronization inside next_item
        const uint32_t jn = gbk::next_item(&s.ctr->work_check, &s_j[buf ^ 1u]);
        if (jn < items && tid == 0) sp_stage(s, win + (buf ^ 1u) * kK * s.rw, &s_bar[buf ^ 1u], jn / kClassBlocks);
        bool ok = gbk::mbar_wait(&s_bar[buf], (phase >> buf) & 1u);
        if (!ok) {
            atomicOr(&s.ctr->err, kErrStaging);
            ok = gbk::mbar_wait(&s_bar[buf], (phase >> buf) & 1u);
        }
        phase ^= 1u << buf;
        const uint32_t c = j / kClassBlocks, cb = j - c * kClassBlocks;
        const uint32_t *w0 = win + buf * kK * s.rw;
        const uint32_t cr1 = min(kHalfM, (cb + 1) * kClassBlock);
        // a chunk inside [start, limit] for every even class needs no
        // per-class range: the latest first even is class 0's, the earliest
        // last even class M - 2's
        const uint64_t ci0 = uint64_t(c) * kChunkEvens;
        const uint64_t ilo_max = s.start > s.N ? (s.start - s.N + kM - 1) / kM : 0;
        const uint64_t top = s.N + kM - 2;
        const uint64_t ihi_min = s.limit >= top ? min(uint64_t(s.dl), (s.limit - top) / kM + 1) : 0;
        const bool interior = ilo_max <= ci0 && ihi_min >= ci0 + kChunkEvens;
        for (uint32_t q0 = cb * kClassBlock + warp; ok && q0 < cr1; q0 += 32 * kCheckWarps) {
            // the group ranges of the warp's next 32 classes, one per lane
            const uint32_t mine = q0 + lane * kCheckWarps;
            uint32_t lg0 = 0, lg1 = 0;
            if (mine < cr1) {
                lg0 = __ldg(goff + mine);
                lg1 = lg0 + min(__ldg(goff + mine + 1) - lg0, s.group_cap);
            }
            const uint32_t nt = min(32u, (cr1 - q0 + kCheckWarps - 1) / kCheckWarps);
            for (uint32_t tj = 0; tj < nt; ++tj) {
                const uint32_t cr = q0 + tj * kCheckWarps;
                const uint32_t g0 = __shfl_sync(~0u, lg0, tj), g1 = __shfl_sync(~0u, lg1, tj);
                uint32_t f[kV];
                if (interior) {
#pragma unroll
                    for (uint32_t v = 0; v < kV; ++v) f[v] = 0u;
                    nevens += 32 * kV;
                } else {
                    // the class's valid evens: i in [ilo, ihi)
                    const uint64_t base = s.N + 2 * cr;
                    uint64_t ilo = 0, ihi = 0;
                    if (s.limit >= base) {
                        ihi = min(uint64_t(s.dl), (s.limit - base) / kM + 1);
                        ilo = s.start > base ? (s.start - base + kM - 1) / kM : 0;
                    }
                    uint32_t all = ~0u;
#pragma unroll
                    for (uint32_t v = 0; v < kV; ++v) {
                        const uint64_t i0 = 32ull * (uint64_t(c) * kChunkWords + 32 * v + lane);
                        const uint32_t lo = ilo > i0 ? uint32_t(min(ilo - i0, uint64_t(32))) : 0u;
                        const uint32_t hi = ihi > i0 ? uint32_t(min(ihi - i0, uint64_t(32))) : 0u;
                        const uint32_t valid = hi > lo ? low_bits(hi) & ~low_bits(lo) : 0u;
                        nevens += __popc(valid);
                        f[v] = ~valid;
                        all &= f[v];
                    }
                    if (__all_sync(~0u, all == ~0u)) continue;
                }
                // the groups in plan order, 32 entries per coalesced load
                uint32_t g = g0;
                bool done = false;
                while (!done && g < g1) {
                    const uint32_t ng = min(32u, g1 - g);
                    uint2 le = make_uint2(0u, 0u);
                    if (lane < ng) le = __ldg(groups + g + lane);
                    uint32_t u = 0;
                    while (u < ng) {
                        const uint32_t ex = __shfl_sync(~0u, le.x, u), ey = __shfl_sync(~0u, le.y, u);
                        ++u;
                        const uint32_t *row = w0 + entry_k(ex) * s.rw + entry_o(ex) + lane;
                        uint32_t a[kV], b[kV];
#pragma unroll
                        for (uint32_t v = 0; v < kV; ++v) {
                            a[v] = row[32 * v];
                            b[v] = row[32 * v + 1];
                        }
                        // two candidates per step
                        const uint32_t np = (entry_n(ex) + 1) >> 1;
                        uint32_t y = ey;
#pragma unroll
                        for (uint32_t jp = 0; jp < (kEntryMax + 1) / 2; ++jp)
                            if (jp < np) {
                                const uint32_t y2 = y >> 5;
#pragma unroll
                                for (uint32_t v = 0; v < kV; ++v)
                                    f[v] |= __funnelshift_r(a[v], b[v], y) | __funnelshift_r(a[v], b[v], y2);
                                y >>= 10;
                            }
                        uint32_t all = f[0];
#pragma unroll
                        for (uint32_t v = 1; v < kV; ++v) all &= f[v];
                        if (__all_sync(~0u, all == ~0u)) {
                            done = true;
                            break;
                        }
                    }
                    g += u;
                }
                ngroups += g - g0;
#pragma unroll
                for (uint32_t v = 0; v < kV; ++v)
                    if (f[v] != ~0u) {
                        const uint32_t slot = atomicAdd(&s.ctr->npend, 1u);
                        if (slot < kPendCap) pend[slot] = make_uint4(cr, c * kChunkWords + 32 * v + lane, ~f[v], 0u);
                    }
            }
        }
        j = jn;
        buf ^= 1u;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) nevens += __shfl_down_sync(~0u, nevens, o);
    if (lane == 0) {
        atomicAdd(&s.ctr->evens, nevens);
        atomicAdd(&s.ctr->groups, ngroups);
    }
}

// per even: the first candidate in plan order with its map bit set (0: none)
__global__ void __launch_bounds__(256) k_sp_witness(SpSeg s, uint64_t start, uint32_t count, const uint2 *groups,
                                                    const uint32_t *goff, uint32_t *out)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count) return;
    const uint64_t off = start + 2ull * j - s.N;
    const uint32_t r = uint32_t(off % kM);
    const uint64_t i = off / kM;
    const uint32_t cr = r >> 1;
    const uint32_t g0 = goff[cr], g1 = g0 + min(goff[cr + 1] - g0, s.group_cap);
    uint32_t p = 0;
    for (uint32_t g = g0; g < g1 && !p; ++g) {
        const uint2 e = groups[g];
        const uint32_t k = entry_k(e.x), o = entry_o(e.x), n = entry_n(e.x);
        for (uint32_t q = 0; q < n; ++q) {
            const uint32_t U = 32 * o + ((e.y >> (5 * q)) & 31u);
            const uint64_t t = i + U;
            if ((s.map[size_t(k) * s.stride + (t >> 5)] >> (t & 31)) & 1u) {
                const uint32_t ck = s.c[k];
                const uint32_t a = s.tb - U - (r < ck ? 1u : 0u);
                p = (r + kM - ck) % kM + kM * a;
                break;
            }
        }
    }
    out[j] = p;
}

}  // namespace gbs

using namespace gbs;

struct gbc_sparse {
    gbc_sparse_config cfg{};
    std::string err;
    uint32_t tb = 0, dlt = 0, rw = 0, stride = 0, tiles_max = 0, pmax = 0;
    uint32_t c[kK] = {};
    uint64_t qbound = 0;                   // sieving primes up to isqrt(limit + M)
    std::vector<uint2> groups;             // plan entries (entry_k / entry_o / entry_n, packed offsets)
    std::vector<uint32_t> goff;            // kHalfM + 1 group offsets
    uint32_t *d_primes = nullptr;          // sieving primes >= 17
    uint32_t nprimes = 0, nsmall = 0, nwarp = 0;
    uint16_t *d_inv = nullptr;
    uint32_t *d_xf = nullptr;
    uint2 *d_groups = nullptr;
    uint32_t *d_goff = nullptr;
    uint32_t *d_map = nullptr;
    uint32_t *d_out = nullptr;             // witness output
    uint32_t out_cap = 0;
    SpCtr *d_ctr = nullptr;
    uint4 *d_pend = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {};
    int sms = 0, check_ctas = 0;
    std::vector<uint64_t> pending;         // evens the last verify left to the CPU
};

namespace {

int sp_fail(gbc_sparse *sp, int code, const std::string &msg)
{
    if (sp) sp->err = msg;
    return code;
}

#define SPCK(call)                                                                                  \
    do {                                                                                            \
        const cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                      \
            return sp_fail(sp, GBC_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
    } while (0)

uint64_t isqrt_u64(uint64_t n)
{
    uint64_t r = 0;
    for (int b = 31; b >= 0; --b) {
        const uint64_t t = r | (1ull << b);
        if (t <= n / t) r = t;
    }
    return r;
}

uint32_t gcd_u32(uint32_t a, uint32_t b)
{
    while (b) {
        const uint32_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

bool unit_mod_m(uint32_t x) { return gcd_u32(x % kM, kM) == 1; }

// x with x = a_j (mod m_j) for the pairwise coprime moduli, by search over
// the progression of the first ones (the moduli are tiny)
uint32_t crt(const uint32_t *a, const uint32_t *m, int n)
{
    uint32_t x = a[0] % m[0], mod = m[0];
    for (int j = 1; j < n; ++j) {
        while (x % m[j] != a[j] % m[j]) x += mod;
        mod *= m[j];
    }
    return x;
}

// Twelve residues mod 30030 that reach every even class. Six are 1 and six
// 2 (mod 3); within each six the residues mod 7, 11 and 13 are pairwise
// distinct and each residue mod 5 appears at most twice. For an even class
// r take the six whose residue mod 3 differs from r's (any six when 3 | r):
// at most two share r's residue mod 5 and at most one each its residue mod
// 7, 11 and 13, so at least one of the six differs from r modulo every odd
// prime of M, i.e. r - c is a unit. (check_cover proves it again.)
void make_residues(uint32_t *c)
{
    static const uint32_t a5[2][6] = {{1, 2, 3, 4, 1, 2}, {3, 4, 1, 2, 3, 4}};
    const uint32_t mods[5] = {3, 5, 7, 11, 13};
    for (uint32_t h = 0; h < 2; ++h)
        for (uint32_t j = 0; j < 6; ++j) {
            const uint32_t a[5] = {h + 1, a5[h][j], h ? 6 - j : j + 1, h ? j + 5 : j + 1, h ? 2 * j + 2 : 2 * j + 1};
            uint32_t x = crt(a, mods, 5);
            if (!(x & 1)) x += kHalfM;
            c[6 * h + j] = x;
        }
    std::sort(c, c + kK);
}

bool check_cover(const uint32_t *c, uint32_t *bad)
{
    for (uint32_t r = 0; r < kM; r += 2) {
        bool any = false;
        for (uint32_t k = 0; k < kK && !any; ++k) any = unit_mod_m(r + kM - c[k]);
        if (!any) {
            *bad = r;
            return false;
        }
    }
    return true;
}

// x^-1 mod M for units x, 0 otherwise
std::vector<uint16_t> inverse_table()
{
    std::vector<uint16_t> inv(kM, 0);
    for (uint32_t x = 1; x < kM; ++x) {
        if (!unit_mod_m(x)) continue;
        int64_t r0 = kM, r1 = x, s0 = 0, s1 = 1;
        while (r1) {
            const int64_t q = r0 / r1;
            int64_t t = r0 - q * r1;
            r0 = r1;
            r1 = t;
            t = s0 - q * s1;
            s0 = s1;
            s1 = t;
        }
        inv[x] = uint16_t(((s0 % int64_t(kM)) + kM) % kM);
    }
    return inv;
}

// Candidate p of even class r and map class k at offset U.
uint32_t decode(uint32_t r, uint32_t ck, uint32_t tb, uint32_t U)
{
    const uint32_t a = tb - U - (r < ck ? 1u : 0u);
    return (r + kM - ck) % kM + kM * a;
}

// The checker plan: per even class r, the candidates p <= pmax of every
// usable class k grouped by (k, window word o = U / 32), the fullest groups
// first (ties: k, then o), each group stored as entries of up to six
// offsets in ascending order. Classes in parallel.
void build_plan(gbc_sparse *sp, const std::vector<uint8_t> &isp)
{
    const uint32_t tb = sp->tb, ow = tb / 32 + 1;
    std::vector<std::vector<uint2>> per(kHalfM);
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    std::atomic<uint32_t> next{0};
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&] {
            std::vector<uint32_t> mask(size_t(kK) * ow);
            for (;;) {
                const uint32_t cr = next.fetch_add(64);
                if (cr >= kHalfM) break;
                for (uint32_t x = cr; x < std::min(kHalfM, cr + 64); ++x) {
                    const uint32_t r = 2 * x;
                    std::fill(mask.begin(), mask.end(), 0u);
                    for (uint32_t k = 0; k < kK; ++k) {
                        const uint32_t ck = sp->c[k], s0 = (r + kM - ck) % kM;
                        if (!unit_mod_m(s0)) continue;
                        for (uint64_t p = s0, a = 0; p <= sp->pmax; p += kM, ++a) {
                            if (!isp[p]) continue;
                            const uint32_t U = tb - uint32_t(a) - (r < ck ? 1u : 0u);
                            mask[size_t(k) * ow + U / 32] |= 1u << (U % 32);
                        }
                    }
                    std::vector<uint2> g;
                    for (uint32_t k = 0; k < kK; ++k)
                        for (uint32_t o = 0; o < ow; ++o)
                            if (mask[size_t(k) * ow + o]) g.push_back(make_uint2(k | o << 4, mask[size_t(k) * ow + o]));
                    std::stable_sort(g.begin(), g.end(),
                                     [](uint2 u, uint2 v) { return __builtin_popcount(u.y) > __builtin_popcount(v.y); });
                    // each group as entries of up to kEntryMax offsets, ascending
                    for (const uint2 &e : g) {
                        uint32_t sh[32], n = 0;
                        for (uint32_t m = e.y; m; m &= m - 1) sh[n++] = uint32_t(__builtin_ctz(m));
                        for (uint32_t i = 0; i < n; i += kEntryMax) {
                            const uint32_t c = std::min(kEntryMax, n - i);
                            uint32_t y = 0;
                            for (uint32_t q = 0; q < c; ++q) y |= sh[i + q] << (5 * q);
                            if (c & 1) y |= sh[i + c - 1] << (5 * c);
                            per[x].push_back(make_uint2(e.x | c << 12, y));
                        }
                    }
                }
            }
        });
    for (auto &x : th) x.join();
    sp->goff.assign(kHalfM + 1, 0);
    sp->groups.clear();
    for (uint32_t x = 0; x < kHalfM; ++x) {
        sp->goff[x] = uint32_t(sp->groups.size());
        sp->groups.insert(sp->groups.end(), per[x].begin(), per[x].end());
    }
    sp->goff[kHalfM] = uint32_t(sp->groups.size());
}

// every plan entry decodes to a prime <= pmax of a usable class, with an
// offset inside the window [0, TB]
bool validate_plan(const gbc_sparse *sp, const std::vector<uint8_t> &isp, std::string *why)
{
    for (uint32_t x = 0; x < kHalfM; ++x) {
        const uint32_t r = 2 * x;
        for (uint32_t g = sp->goff[x]; g < sp->goff[x + 1]; ++g) {
            const uint2 e = sp->groups[g];
            const uint32_t k = entry_k(e.x), o = entry_o(e.x), n = entry_n(e.x);
            if (k >= kK || n == 0 || n > kEntryMax || (e.x >> 15) ||
                ((n & 1) && ((e.y >> (5 * n)) & 31u) != ((e.y >> (5 * (n - 1))) & 31u))) {
                *why = "entry layout";
                return false;
            }
            for (uint32_t q = 0; q < n; ++q) {
                const uint32_t U = 32 * o + ((e.y >> (5 * q)) & 31u);
                const uint32_t ck = sp->c[k];
                if (U > sp->tb || U + (r < ck ? 1u : 0u) > sp->tb) {
                    *why = "offset outside the window";
                    return false;
                }
                const uint32_t p = decode(r, ck, sp->tb, U);
                if (p > sp->pmax || !isp[p] || !unit_mod_m(p) || !unit_mod_m(r + kM - ck)) {
                    *why = "candidate " + std::to_string(p) + " of even class " + std::to_string(r);
                    return false;
                }
            }
        }
    }
    return true;
}

SpSeg make_seg(const gbc_sparse *sp, uint64_t N, uint32_t dl, uint64_t start, uint64_t limit)
{
    SpSeg s{};
    s.N = N;
    s.Q = N - uint64_t(kM) * sp->tb;
    s.start = start;
    s.limit = limit;
    s.dl = dl;
    s.tb = sp->tb;
    s.T = dl + sp->tb;
    s.chunks = (dl + kChunkEvens - 1) / kChunkEvens;
    const uint64_t need = uint64_t(s.chunks) * kChunkEvens + uint64_t(sp->rw) * 32;
    s.tiles = uint32_t((std::max<uint64_t>(need, s.T) + kTileBits - 1) / kTileBits);
    s.stride = sp->stride;
    s.rw = sp->rw;
    s.group_cap = sp->cfg.group_cap ? sp->cfg.group_cap : ~0u;
    s.map = sp->d_map;
    s.ctr = sp->d_ctr;
    std::memcpy(s.c, sp->c, sizeof s.c);
    return s;
}

// the map of segment s: first bits, tiles, large primes, set-bit count
int build_map(gbc_sparse *sp, const SpSeg &s)
{
    SPCK(cudaMemsetAsync(sp->d_ctr, 0, sizeof(SpCtr), sp->st));
    SPCK(cudaEventRecord(sp->ev[0], sp->st));
    if (sp->nsmall) {
        k_sp_first<<<(sp->nsmall + 255) / 256, 256, 0, sp->st>>>(s, sp->d_primes, sp->nsmall, sp->d_inv, sp->d_xf);
        SPCK(cudaGetLastError());
    }
    k_sp_tile<<<sp->sms, 1024, kTileWords * 4, sp->st>>>(s, sp->d_primes, sp->nsmall, sp->nwarp, sp->d_xf);
    SPCK(cudaGetLastError());
    SPCK(cudaEventRecord(sp->ev[1], sp->st));
    if (sp->nprimes > sp->nsmall) {
        k_sp_large<<<sp->sms * 8, 256, 0, sp->st>>>(s, sp->d_primes, sp->nsmall, sp->nprimes, sp->d_inv);
        SPCK(cudaGetLastError());
    }
    k_sp_popc<<<sp->sms * 4, 256, 0, sp->st>>>(s);
    SPCK(cudaGetLastError());
    SPCK(cudaEventRecord(sp->ev[2], sp->st));
    return GBC_OK;
}

int sp_sync(gbc_sparse *sp)
{
    SPCK(cudaStreamSynchronize(sp->st));
    return GBC_OK;
}

float ev_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

extern "C" int gbc_sparse_create(const gbc_sparse_config *cfg_in, gbc_sparse **out)
{
    if (!cfg_in || !out) return GBC_E_ARG;
    *out = nullptr;
    gbc_sparse *sp = new gbc_sparse();
    sp->cfg = *cfg_in;
    gbc_sparse_config &cfg = sp->cfg;
    if (!cfg.dlt_log2) cfg.dlt_log2 = 26;
    if (!cfg.pmax) cfg.pmax = 40000000;
    int rc = GBC_OK;
    if (cfg.dlt_log2 < 12 || cfg.dlt_log2 > 26) rc = sp_fail(sp, GBC_E_ARG, "dlt_log2 outside [12, 26]");
    else if (cfg.pmax < 100000 || cfg.pmax > 200000000) rc = sp_fail(sp, GBC_E_ARG, "pmax outside [1e5, 2e8]");
    else if (cfg.limit < 1000000 || cfg.limit > GBC_MAX_LIMIT) rc = sp_fail(sp, GBC_E_ARG, "limit out of range");
    if (rc) {
        *out = sp;
        return rc;
    }
    sp->dlt = 1u << cfg.dlt_log2;
    sp->pmax = cfg.pmax;
    sp->tb = (cfg.pmax + kM - 1) / kM + 2;
    sp->rw = (kChunkWords + sp->tb / 32 + 2 + 3) & ~3u;
    {
        const uint64_t bits = uint64_t(sp->dlt) + kChunkEvens + uint64_t(sp->rw) * 32 + sp->tb;
        sp->tiles_max = uint32_t((bits + kTileBits - 1) / kTileBits);
        sp->stride = sp->tiles_max * kTileWords;
    }
    make_residues(sp->c);
    uint32_t bad = 0;
    if (!check_cover(sp->c, &bad)) {
        *out = sp;
        return sp_fail(sp, GBC_E_STATE, "residues reach no class for even class " + std::to_string(bad));
    }
    // candidates: the primes <= pmax
    std::vector<uint8_t> isp(size_t(cfg.pmax) + 1, 0);
    for (uint32_t p : gbh_odd_primes_upto(cfg.pmax)) isp[p] = 1;
    build_plan(sp, isp);
    std::string why;
    if (!validate_plan(sp, isp, &why)) {
        *out = sp;
        return sp_fail(sp, GBC_E_STATE, "sparse plan failed validation: " + why);
    }
    if (cfg.host_only) {
        *out = sp;
        return GBC_OK;
    }
    // sieving primes 17 .. isqrt(limit + M)
    sp->qbound = isqrt_u64(cfg.limit + kM) + 1;
    std::vector<uint32_t> pr = gbh_cached_primes(std::max<uint64_t>(sp->qbound, 17));
    pr.erase(pr.begin(), std::lower_bound(pr.begin(), pr.end(), 17u));
    sp->nprimes = uint32_t(pr.size());
    sp->nsmall = uint32_t(std::lower_bound(pr.begin(), pr.end(), kSplit) - pr.begin());
    sp->nwarp = uint32_t(std::lower_bound(pr.begin(), pr.end(), kWarpPrime) - pr.begin());
    const std::vector<uint16_t> inv = inverse_table();

    *out = sp;
    SPCK(cudaSetDevice(cfg.device));
    cudaDeviceProp prop{};
    SPCK(cudaGetDeviceProperties(&prop, cfg.device));
    sp->sms = prop.multiProcessorCount;
    SPCK(cudaStreamCreateWithFlags(&sp->st, cudaStreamNonBlocking));
    for (auto &e : sp->ev) SPCK(cudaEventCreate(&e));
    SPCK(cudaMalloc(&sp->d_primes, std::max<size_t>(pr.size(), 1) * 4));
    if (!pr.empty()) SPCK(cudaMemcpy(sp->d_primes, pr.data(), pr.size() * 4, cudaMemcpyHostToDevice));
    SPCK(cudaMalloc(&sp->d_inv, kM * 2));
    SPCK(cudaMemcpy(sp->d_inv, inv.data(), kM * 2, cudaMemcpyHostToDevice));
    SPCK(cudaMalloc(&sp->d_xf, std::max<size_t>(size_t(kK) * sp->nsmall, 1) * 4));
    SPCK(cudaMalloc(&sp->d_groups, std::max<size_t>(sp->groups.size(), 1) * sizeof(uint2)));
    if (!sp->groups.empty())
        SPCK(cudaMemcpy(sp->d_groups, sp->groups.data(), sp->groups.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    SPCK(cudaMalloc(&sp->d_goff, (kHalfM + 1) * 4));
    SPCK(cudaMemcpy(sp->d_goff, sp->goff.data(), (kHalfM + 1) * 4, cudaMemcpyHostToDevice));
    SPCK(cudaMalloc(&sp->d_map, size_t(kK) * sp->stride * 4));
    SPCK(cudaMemset(sp->d_map, 0, size_t(kK) * sp->stride * 4));
    SPCK(cudaMalloc(&sp->d_ctr, sizeof(SpCtr)));
    SPCK(cudaMalloc(&sp->d_pend, size_t(kPendCap) * sizeof(uint4)));
    SPCK(cudaFuncSetAttribute(k_sp_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTileWords * 4)));
    const int csmem = int(2 * kK * sp->rw * 4);
    SPCK(cudaFuncSetAttribute(k_sp_check, cudaFuncAttributeMaxDynamicSharedMemorySize, csmem));
    int occ = 0;
    SPCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sp_check, kCheckThreads, csmem));
    sp->check_ctas = sp->sms * std::max(1, occ);
    return GBC_OK;
}

extern "C" void gbc_sparse_destroy(gbc_sparse *sp)
{
    if (!sp) return;
    if (sp->st) cudaStreamSynchronize(sp->st);
    cudaFree(sp->d_primes);
    cudaFree(sp->d_inv);
    cudaFree(sp->d_xf);
    cudaFree(sp->d_groups);
    cudaFree(sp->d_goff);
    cudaFree(sp->d_map);
    cudaFree(sp->d_out);
    cudaFree(sp->d_ctr);
    cudaFree(sp->d_pend);
    for (auto &e : sp->ev)
        if (e) cudaEventDestroy(e);
    if (sp->st) cudaStreamDestroy(sp->st);
    delete sp;
}

extern "C" const char *gbc_sparse_last_error(const gbc_sparse *sp) { return sp ? sp->err.c_str() : "no context"; }

extern "C" int gbc_sparse_geometry(const gbc_sparse *sp, uint32_t *M, uint32_t *K, uint32_t *res, uint32_t *tb,
                                   uint32_t *dlt, uint32_t *pmax)
{
    if (!sp || sp->goff.empty()) return GBC_E_STATE;
    if (M) *M = kM;
    if (K) *K = kK;
    if (res) std::memcpy(res, sp->c, sizeof sp->c);
    if (tb) *tb = sp->tb;
    if (dlt) *dlt = sp->dlt;
    if (pmax) *pmax = sp->pmax;
    return GBC_OK;
}

// the segment at N with dl evens per class lies where the map is exact
static int check_reach(gbc_sparse *sp, uint64_t N, uint32_t dl)
{
    const uint64_t sq = isqrt_u64(sp->cfg.limit + kM) + 1;
    if (N < uint64_t(kM) * (sp->tb + 1) || N - uint64_t(kM) * (sp->tb + 1) <= sq || N <= sp->pmax)
        return sp_fail(sp, GBC_E_ARG, "start too low for the sparse map (its q must exceed sqrt(limit) and pmax): "
                                      "use the dense path");
    if (dl == 0 || dl > sp->dlt) return sp_fail(sp, GBC_E_ARG, "evens per class outside [1, dlt]");
    if (N + uint64_t(kM) * dl > sp->cfg.limit + kM) return sp_fail(sp, GBC_E_ARG, "segment beyond the context's limit");
    return GBC_OK;
}

extern "C" int gbc_sparse_verify(gbc_sparse *sp, uint64_t start, uint64_t limit, gbc_sparse_result *res)
{
    if (!sp || !sp->d_map) return GBC_E_STATE;
    if (!res) return sp_fail(sp, GBC_E_ARG, "result pointer is NULL");
    std::memset(res, 0, sizeof *res);
    sp->pending.clear();
    if (start & 1) ++start;
    if (limit & 1) --limit;
    if (start > limit) return sp_fail(sp, GBC_E_ARG, "start > limit");
    if (limit > sp->cfg.limit) return sp_fail(sp, GBC_E_ARG, "limit above the context's limit");
    const auto t0 = std::chrono::steady_clock::now();
    const uint64_t D = uint64_t(kM) * sp->dlt;
    const uint64_t N0 = start - start % kM;
    if (int rc = check_reach(sp, N0, 1)) return rc;
    res->evens = (limit - start) / 2 + 1;
    uint64_t checked = 0;
    std::vector<uint4> pend;
    for (uint64_t N = N0; N <= limit; N += D) {
        const uint32_t dl = uint32_t(std::min<uint64_t>(sp->dlt, (limit - N) / kM + 1));
        if (int rc = check_reach(sp, N, dl)) return rc;
        const SpSeg s = make_seg(sp, N, dl, start, limit);
        if (s.tiles > sp->tiles_max) return sp_fail(sp, GBC_E_STATE, "segment larger than the map");
        if (int rc = build_map(sp, s)) return rc;
        k_sp_check<<<sp->check_ctas, kCheckThreads, 2 * kK * sp->rw * 4, sp->st>>>(s, sp->d_groups, sp->d_goff,
                                                                                 sp->d_pend);
        SPCK(cudaGetLastError());
        SPCK(cudaEventRecord(sp->ev[3], sp->st));
        SpCtr ctr{};
        SPCK(cudaMemcpyAsync(&ctr, sp->d_ctr, sizeof ctr, cudaMemcpyDeviceToHost, sp->st));
        if (int rc = sp_sync(sp)) return rc;
        res->ms_sieve += ev_ms(sp->ev[0], sp->ev[1]);
        res->ms_large += ev_ms(sp->ev[1], sp->ev[2]);
        res->ms_check += ev_ms(sp->ev[2], sp->ev[3]);
        res->map_primes += ctr.map_primes;
        res->groups += ctr.groups;
        res->segments += 1;
        checked += ctr.evens;
        if (ctr.err) return sp_fail(sp, GBC_E_DEVICE, "device error flags " + std::to_string(ctr.err));
        if (ctr.npend > kPendCap)
            return sp_fail(sp, GBC_E_OVERFLOW, "pending words " + std::to_string(ctr.npend) + " beyond the list");
        if (ctr.npend) {
            pend.resize(ctr.npend);
            SPCK(cudaMemcpy(pend.data(), sp->d_pend, size_t(ctr.npend) * sizeof(uint4), cudaMemcpyDeviceToHost));
            for (const uint4 &e : pend)
                for (uint32_t m = e.z; m; m &= m - 1) {
                    const uint64_t i = 32ull * e.y + uint32_t(__builtin_ctz(m));
                    sp->pending.push_back(N + 2ull * e.x + uint64_t(kM) * i);
                }
        }
    }
    if (checked != res->evens)
        return sp_fail(sp, GBC_E_DEVICE, "checker covered " + std::to_string(checked) + " evens of " +
                                             std::to_string(res->evens));
    std::sort(sp->pending.begin(), sp->pending.end());
    res->pending = sp->pending.size();
    for (uint64_t n : sp->pending)
        if (!gbc_pn_exact(n)) return sp_fail(sp, GBC_E_STATE, "no Goldbach pair for " + std::to_string(n));
    res->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GBC_OK;
}

extern "C" int gbc_sparse_pending(const gbc_sparse *sp, uint64_t *out, uint64_t cap, uint64_t *count)
{
    if (!sp) return GBC_E_STATE;
    if (count) *count = sp->pending.size();
    if (out)
        for (uint64_t j = 0; j < cap && j < sp->pending.size(); ++j) out[j] = sp->pending[j];
    return GBC_OK;
}

extern "C" int gbc_sparse_map(gbc_sparse *sp, uint64_t n0, uint32_t dl, uint32_t *out, uint64_t out_words)
{
    if (!sp || !sp->d_map) return GBC_E_STATE;
    if (n0 % kM) return sp_fail(sp, GBC_E_ARG, "n0 is not a multiple of M");
    if (int rc = check_reach(sp, n0, dl)) return rc;
    const uint32_t rows = (dl + sp->tb + 31) / 32;
    if (!out || out_words < uint64_t(kK) * rows) return sp_fail(sp, GBC_E_ARG, "output smaller than K rows");
    const SpSeg s = make_seg(sp, n0, dl, n0, n0 + uint64_t(kM) * dl - 2);
    if (int rc = build_map(sp, s)) return rc;
    SPCK(cudaMemcpy2DAsync(out, size_t(rows) * 4, sp->d_map, size_t(sp->stride) * 4, size_t(rows) * 4, kK,
                           cudaMemcpyDeviceToHost, sp->st));
    return sp_sync(sp);
}

extern "C" int gbc_sparse_witness(gbc_sparse *sp, uint64_t start, uint32_t count, uint32_t *p_out)
{
    if (!sp || !sp->d_map) return GBC_E_STATE;
    if (!count) return GBC_OK;
    if (!p_out || (start & 1)) return sp_fail(sp, GBC_E_ARG, "odd start or NULL output");
    const uint64_t N = start - start % kM, last = start + 2ull * (count - 1);
    const uint64_t dl64 = (last - N) / kM + 1;
    if (dl64 > sp->dlt) return sp_fail(sp, GBC_E_ARG, "evens beyond one segment");
    if (int rc = check_reach(sp, N, uint32_t(dl64))) return rc;
    const SpSeg s = make_seg(sp, N, uint32_t(dl64), start, last);
    if (int rc = build_map(sp, s)) return rc;
    if (count > sp->out_cap) {
        cudaFree(sp->d_out);
        sp->d_out = nullptr;
        sp->out_cap = 0;
        SPCK(cudaMalloc(&sp->d_out, size_t(count) * 4));
        sp->out_cap = count;
    }
    k_sp_witness<<<(count + 255) / 256, 256, 0, sp->st>>>(s, start, count, sp->d_groups, sp->d_goff, sp->d_out);
    SPCK(cudaGetLastError());
    SPCK(cudaMemcpyAsync(p_out, sp->d_out, size_t(count) * 4, cudaMemcpyDeviceToHost, sp->st));
    return sp_sync(sp);
}

extern "C" int gbc_sparse_plan(const gbc_sparse *sp, uint32_t r, uint32_t *p_out, uint32_t *group_out, int cap)
{
    if (!sp || sp->goff.empty()) return GBC_E_STATE;
    if ((r & 1) || r >= kM) return GBC_E_ARG;
    const uint32_t x = r / 2;
    int n = 0;
    for (uint32_t g = sp->goff[x]; g < sp->goff[x + 1]; ++g) {
        const uint2 e = sp->groups[g];
        const uint32_t k = entry_k(e.x), o = entry_o(e.x), c = entry_n(e.x);
        for (uint32_t q = 0; q < c; ++q, ++n) {
            if (n >= cap) continue;
            const uint32_t U = 32 * o + ((e.y >> (5 * q)) & 31u);
            if (p_out) p_out[n] = decode(r, sp->c[k], sp->tb, U);
            if (group_out) group_out[n] = g - sp->goff[x];
        }
    }
    return n;
}
