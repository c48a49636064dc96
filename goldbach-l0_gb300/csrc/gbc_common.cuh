// gbc_common.cuh -- types and device helpers shared by the sieve, checker
// and count kernels of the dense Goldbach verify path.
//
// Layout of a batch's class map (HBM-resident, one per slot):
//   8 class arrays, one per residue u_k in {1, 7, 11, 13, 17, 19, 23, 29}
//   (mod 30); bit t of array k <-> q = base + 30 t + u_k, base a multiple
//   of 30. Array k holds words [k * wpc, (k + 1) * wpc) of u32; bit t is
//   bit (t & 31) of word t >> 5. A set bit means q is prime. The layout
//   keeps the reference's mod-30 class map (include/host_math.hpp:63-78)
//   with the class phases fixed to 0 by aligning base to 30.
#pragma once
#include <cstdint>

#include "../../include/gbc.h"

namespace gbk {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kNumGroups = 7;         // small-prime pattern groups (primes 7..67)
constexpr uint32_t kFirstSievePrime = 71;
constexpr uint32_t kSkip1 = 1001;     // 7 * 11 * 13: large-prime multiplier skip
constexpr uint32_t kSkip2 = 7429;     // 17 * 19 * 23

// u_k, the residue of class array k
__host__ __device__ __forceinline__ uint32_t unit30(uint32_t k)
{
    // bytes, low to high: 1, 7, 11, 13, 17, 19, 23, 29
    return uint32_t((0x1D1713110D0B0701ull >> (8 * k)) & 0xFF);
}

// class array index of a residue mod 30, or 8 when it is not coprime to 30
__host__ __device__ __forceinline__ uint32_t class_of(uint32_t u)
{
    uint32_t c = 8;
    for (uint32_t k = 0; k < 8; ++k)
        if (unit30(k) == u) c = k;
    return c;
}

// 30^-1 mod p for a prime p > 5: (j p + 1) / 30 with j p = -1 (mod 30)
__host__ __device__ __forceinline__ uint32_t inv30_mod(uint32_t p)
{
    const uint32_t s = p % 30;
    // s^-1 mod 30 for the units: 1->1 7->13 11->11 13->7 17->23 19->19 23->17 29->29
    uint32_t inv;
    switch (s) {
    case 1: inv = 1; break;
    case 7: inv = 13; break;
    case 11: inv = 11; break;
    case 13: inv = 7; break;
    case 17: inv = 23; break;
    case 19: inv = 19; break;
    case 23: inv = 17; break;
    default: inv = 29; break;
    }
    const uint32_t j = (30 - inv) % 30;
    return uint32_t((uint64_t(j) * p + 1) / 30);
}

// One batch: its map and the sieving primes that reach it.
struct BatchParams {
    uint64_t base;            // multiple of 30
    uint64_t qmax;            // largest q the batch needs exact
    uint32_t nblk;            // bits per class array in use
    uint32_t wpc;             // words per class array (stride)
    uint32_t *map;            // 8 * wpc words
    const uint32_t *primes;   // odd primes ascending
    const uint32_t *magic;    // floor(2^32 / p) for primes[0 .. n_mid)
    uint32_t *xfirst;         // 8 * n_mid first class bits of this batch
    uint32_t i0;              // index of the first tile-sieve prime (71)
    uint32_t i_warp;          // primes [i0, i_warp): warp-cooperative marking
    uint32_t n_mid;           // primes [i_warp, n_mid): one thread per prime
    uint32_t n_all;           // primes [n_mid, n_all): large-prime kernel
    uint32_t tile_log2;
    uint32_t tiles_pc;        // tiles per class array
    const uint32_t *pat;      // pattern words of the groups, back to back
    const uint32_t *skip_tab; // bit tables: multipliers to skip (1001 then 7429 bits)
    const uint16_t *inv_tab;  // inverses mod 1001 then mod 7429 (0: none)
    uint32_t *err;            // device error word of the slot
    // prime-multiplier table: primes [n_hl, n_all) mark only p m with m prime
    uint32_t n_hl;            // first hit-listed prime (n_all: none)
    const uint32_t *mtab;     // bit k of byte i <-> m = m0 + 30 i + u_k is prime
    uint64_t m0, m1;          // the table covers m in [m0, m1]
};

struct GroupInfo {
    uint32_t P[kNumGroups];       // period (product of the group's primes)
    uint32_t off[kNumGroups];     // word offset of the group's pattern
    uint32_t inv30[kNumGroups];   // 30^-1 mod P
    uint32_t words;               // total pattern words
};

// One segment of a batch, as the checker and count kernels see it.
struct SegParams {
    uint64_t seg_start, seg_end;  // evens, inclusive
    uint64_t cnt_lo, cnt_hi;      // counted primes (odd q)
    uint64_t twin_hi;             // largest counted lower twin prime
    uint64_t hash_lo, hash_hi;    // hashed q range
    uint32_t flags;
    uint32_t low;                 // seg_start < 9788: the generic per-even checker
    gbc_segment_result *res;      // device result of this segment
    uint16_t *pn;                 // per-even p(n) or nullptr
    uint32_t sampled;             // 1: exact p(n) of every even; 0: funnel verify + exact tail
    uint2 *pend;                  // phase-A misses: (class r / 2 << 27 | word, unresolved bits)
    uint32_t pend_cap;
};

// Candidate tables of the checker (uploaded once per context).
struct CheckTables {
    const uint16_t *cand;   // odd primes 3..9781
    const uint16_t *list;   // per class r / 2: useful candidate indices ascending
    uint32_t off[GBC_NCLASS];
    uint32_t cnt[GBC_NCLASS];
    uint32_t ridge_min;     // evens with p(n) >= ridge_min are listed with their p(n)
};

// Funnel plan of the verify (phase A) checker and the ascending rest lists
// of its exact continuation (phase B), per class r / 2.
struct VerifyTables {
    const uint16_t *cand;
    const uint32_t *fun;    // funnel: candidate index of its first member | mask << 16 (bit d: p + 30 d)
    const uint16_t *rest;   // candidates no funnel tests, ascending
    uint32_t fun_off[GBC_NCLASS], fun_cnt[GBC_NCLASS];
    uint32_t rest_off[GBC_NCLASS], rest_cnt[GBC_NCLASS];
    uint32_t ridge_min;     // evens with p(n) >= ridge_min are listed with their p(n)
};

// device error flags
constexpr uint32_t kErrLeftOverflow = 1u << 0;
constexpr uint32_t kErrTailOverflow = 1u << 1;
constexpr uint32_t kErrGapRange = 1u << 2;
constexpr uint32_t kErrNoPred = 1u << 3;
constexpr uint32_t kErrRetry = 1u << 4;
constexpr uint32_t kErrTable = 1u << 5;   // a multiplier outside the prime-multiplier table
constexpr uint32_t kErrPendOverflow = 1u << 6;
constexpr uint32_t kErrRidgeOverflow = 1u << 7;

// ---------------------------------------------------------------------------
// 64-bit Miller-Rabin in Montgomery form (the GPU retry of evens without a
// witness <= 9781). Deterministic for all u64 with the bases 2..37 (the
// published result of Sorenson and Webster; the reference uses the same
// twelve bases, src/primes.cpp:445-480).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mont_mul(uint64_t a, uint64_t b, uint64_t n, uint64_t nneg_inv)
{
    const uint64_t lo = a * b, hi = __umul64hi(a, b);
    const uint64_t m = lo * nneg_inv;
    const uint64_t mlo = m * n, mhi = __umul64hi(m, n);
    // (a b + m n) / 2^64 = hi + mhi + carry(lo + mlo); lo + mlo = 0 mod 2^64
    const uint64_t carry = (lo != 0) ? 1 : 0;
    (void)mlo;
    uint64_t t = hi + mhi;
    bool over = t < hi;
    const uint64_t t2 = t + carry;
    over = over || (t2 < t);
    t = t2;
    if (over || t >= n) t -= n;
    return t;
}

__device__ inline bool is_prime_u64_dev(uint64_t n)
{
    const uint32_t bases[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (n < 2) return false;
    for (int i = 0; i < 12; ++i)
        if (n % bases[i] == 0) return n == bases[i];
    // n odd, > 37
    uint64_t inv = n;  // Newton: inv = n^-1 mod 2^64
    for (int i = 0; i < 6; ++i) inv *= 2 - n * inv;
    const uint64_t nneg_inv = 0 - inv;
    uint64_t one = (0 - n) % n;  // 2^64 mod n
    uint64_t r2 = one;           // 2^128 mod n by 64 doublings
    for (int i = 0; i < 64; ++i) r2 = (r2 >= n - r2) ? r2 - (n - r2) : r2 + r2;
    const uint64_t mone = n - one;  // -1 in Montgomery form
    uint64_t d = n - 1;
    int s = 0;
    while (!(d & 1)) {
        d >>= 1;
        ++s;
    }
    for (int i = 0; i < 12; ++i) {
        uint64_t a = mont_mul(bases[i], r2, n, nneg_inv);  // a R mod n
        uint64_t x = one;
        for (int b = 63; b >= 0; --b) {
            x = mont_mul(x, x, n, nneg_inv);
            if ((d >> b) & 1) x = mont_mul(x, a, n, nneg_inv);
        }
        if (x == one || x == mone) continue;
        bool comp = true;
        for (int r = 1; r < s; ++r) {
            x = mont_mul(x, x, n, nneg_inv);
            if (x == mone) {
                comp = false;
                break;
            }
        }
        if (comp) return false;
    }
    return true;
}

}  // namespace gbk

// Host-side launchers (defined in the kernel translation units).
namespace gbh {
void launch_xfirst(const gbk::BatchParams &bp, cudaStream_t st);
void launch_tile(const gbk::BatchParams &bp, const gbk::GroupInfo &gi, cudaStream_t st);
int launch_large(const gbk::BatchParams &bp, uint32_t pass_mb, cudaStream_t st);
int launch_hitlist(const gbk::BatchParams &bp, uint32_t pass_mb, cudaStream_t st);
void launch_wheel_bytes(const gbk::BatchParams &bp, uint32_t *out, cudaStream_t st);
void launch_check(const gbk::BatchParams &bp, const gbk::SegParams &sp, const gbk::CheckTables &ct, int sm_count,
                  cudaStream_t st);
void launch_retry(const gbk::SegParams &sp, uint32_t ridge_min, cudaStream_t st);
void launch_verify(const gbk::BatchParams &bp, const gbk::SegParams &sp, const gbk::VerifyTables &vt, int sm_count,
                   cudaStream_t st);
void launch_count(const gbk::BatchParams &bp, const gbk::SegParams &sp, cudaStream_t st);
}  // namespace gbh
