// gbc_common.cuh -- types and device helpers shared by the sieve, checker
// and count kernels of the dense Goldbach verify path.
//
// Layout of a run's class map (HBM-resident; a run is a maximal set of
// consecutive segments of a batch, and each run has its own map in the
// slot's map buffer):
//   8 class arrays, one per residue u_k in {1, 7, 11, 13, 17, 19, 23, 29}
//   (mod 30); bit t of array k <-> q = base + 30 t + u_k, base a multiple
//   of 30. Array k holds words [k * wpc, (k + 1) * wpc) of u32 from the
//   run's map pointer; bit t is bit (t & 31) of word t >> 5. A set bit means
//   q is prime. The layout keeps the reference's mod-30 class map
//   (include/host_math.hpp:63-78) with the class phases fixed to 0 by
//   aligning base to 30.
#pragma once
#include <cstdint>

#include "../../include/gbc.h"

namespace gbk {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kNumGroups = 7;         // small-prime pattern groups (primes 7..67)
constexpr uint32_t kFirstSievePrime = 71;
constexpr uint32_t kWheelM = 1001;    // 7 * 11 * 13: the large-prime multiplier wheel
// the wheel table: per residue the next unit's rank | distance << 10 (1001),
// the 720 unit gaps, the inverses mod 1001 (1001), the inverses mod 17..43
// back to back (240)
constexpr uint32_t kWheelTabWords = 1001 + 720 + 1001 + 240;
constexpr uint32_t kPackGroup = 256;  // packed large primes per group (one warp decodes a group)

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
    uint32_t tile_log2;       // the single-run forms' tiles: 2^tile_log2 bits
    uint32_t tile_bits;       // the batch kernels' tiles: bits per tile, a multiple of 128
    uint32_t tile_rcp;        // ceil(2^32 / tile_bits): t / tile_bits by one multiply and a correction
    uint32_t tiles_pc;        // tiles per class array
    const uint32_t *pat;      // pattern words of the groups, back to back
    const uint16_t *wheel;    // the large primes' multiplier wheel (kWheelTabWords)
    const uint8_t *pk_gap;    // packed large primes [pk_i0, ...): half gaps, 0 at each group start
    const uint32_t *pk_base;  // the first prime of each group of kPackGroup
    uint32_t pk_i0;           // index of the first packed prime
    uint32_t *err;            // device error word of the slot
    // prime-multiplier table: primes [n_hl, n_all) mark only p m with m prime
    uint32_t n_hl;            // first hit-listed prime (n_all: none)
    const uint32_t *mtab;     // bit k of byte i <-> m = m0 + 30 i + u_k is prime
    uint64_t m0, m1;          // the table covers m in [m0, m1]
    uint32_t bm1;             // base mod 1001
    uint8_t bres[8];          // base mod 17, 19, 23, 29, 31, 37, 41, 43
    // binned hit lists (hl_quota and tb_cap both set, in every run of the
    // batch): the runs' class arrays are laid end to end, each from a whole
    // tile, as one virtual array per class (run r's bit t is virtual bit
    // tb_vt0 * tile_bits + t, below 2^31); the harvest files each mark's
    // virtual offset in its (harvest CTA, region bin) quota, bin = class *
    // hl_nreg + (v >> hl_rlog); k_binsort moves them to one bin per virtual
    // tile; the tile kernel clears its tile's marks in shared memory before
    // storing the tile. Marks beyond a quota or a tile bin's capacity go to
    // the overflow list, cleared after the tiles. Otherwise the harvest
    // clears its marks directly, after the tiles.
    uint32_t *hl_buf;         // hl_ctas * hl_nbin * hl_quota offsets
    uint32_t *hl_cnt;         // hl_ctas * hl_nbin counts (capped at the quota when read)
    uint32_t hl_quota, hl_rlog, hl_nreg, hl_ctas;
    uint32_t *tb_buf;         // 8 * tb_tiles tile bins of tb_cap offsets within the tile
    uint32_t *tb_cnt;         // 8 * tb_tiles counts (capped at tb_cap when read)
    uint32_t tb_cap;          // multiple of 32
    uint32_t tb_vt0;          // the run's first virtual tile (0 for a one-run batch)
    uint32_t tb_tiles;        // virtual tiles per class (the batch's tiles_pc summed)
    uint32_t ovf_cap;
    uint2 *ovf_buf;           // (class, virtual bit) of each overflow mark
    uint32_t *ovf_cnt;
    uint32_t spin0;           // try_wait rounds of the first wait on a tile bin's bulk copies (kStageSpin)
};

// t / tile_bits for t < 2^31 (the estimate umulhi(t, rcp) is exact or one
// too high)
__host__ __device__ __forceinline__ uint32_t tile_of(uint32_t t, uint32_t tile_bits, uint32_t rcp)
{
#ifdef __CUDA_ARCH__
    uint32_t q = __umulhi(t, rcp);
#else
    uint32_t q = uint32_t((uint64_t(t) * rcp) >> 32);
#endif
    if (q * tile_bits > t) --q;
    return q;
}

// a batch whose hit lists go through the tile bins (set in every run of it)
__host__ __device__ __forceinline__ bool hl_binned(const BatchParams &bp0)
{
    return bp0.hl_quota != 0 && bp0.tb_cap != 0;
}

struct GroupInfo {
    uint32_t P[kNumGroups];       // period (product of the group's primes)
    uint32_t off[kNumGroups];     // word offset of the group's pattern
    uint32_t inv30[kNumGroups];   // 30^-1 mod P
    uint32_t words;               // total pattern words
};

// Bit and word ranges of one segment for the count kernel (per class k:
// bits [lo, hi] of the ranges).
struct CountRanges {
    uint32_t hash_t[8][2];  // hashed q range
    uint32_t cnt_t[8][2];   // counted primes
    uint32_t twin_t[8][2];  // counted lower twin primes
    uint32_t w_lo, w_hi;    // words covering the hashed range
    uint32_t in_lo, in_hi;  // words inside all three ranges for every class (in_hi < in_lo: none)
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
    uint32_t run;                 // the segment's run (class map) in the batch
    uint32_t vbx;                 // checker CTAs per class of the segment
    uint32_t pad;
    CountRanges cr;
};

// A batch as the persistent kernels see it: a header of counts and the
// per-run and per-segment parameter arrays, all in device memory and
// rewritten for every batch by one host-to-device copy. The pointers are
// fixed for a slot, so one CUDA graph of the whole pipeline, captured once,
// replays every batch.
struct BatchHeader {
    uint32_t nrun, nseg;
    uint32_t tile_items;           // (run, tile, class) items of the tile kernel, tile-major per run
    uint32_t n_mid_max;            // first bits: primes [i0, n_mid_max)
    uint32_t n_mid_min, n_hl_max;  // large primes: [n_mid_min, n_hl_max)
    uint32_t n_hl_min, n_all_max;  // hit-listed primes: [n_hl_min, n_all_max)
    uint32_t chk_vb, ver_vb, cnt_vb; // virtual CTAs of k_check, k_verify, k_count
    uint32_t nlow;                 // segments that need the generic low checker
    // a window of the batch for the per-segment launches of the plain form
    // (launch mode 3; the whole batch otherwise): segments [seg0, nseg) for
    // the kernels that walk segments, class bits [win_b0, win_b1) of run 0
    // for the large primes and the overflow marks (tile-aligned); the item
    // ranges of the other kernels are their work counters' start values
    // and limits
    uint32_t seg0;
    uint32_t win_b0, win_b1;
    uint32_t pad;
    // work counters of the persistent kernels (CTAs take their next item
    // with an atomic add); zero in the host image, so every batch's
    // descriptor copy resets them
    uint32_t work[5];
};

constexpr int kWorkTile = 0, kWorkCheck = 1, kWorkVerify = 2, kWorkCount = 3, kWorkBinsort = 4;
constexpr uint32_t kHlMaxBins = 64;  // region bins of a binned batch (8 classes x up to 8 regions)

struct BatchDesc {
    const BatchHeader *h;
    uint32_t *work;               // h->work, writable
    const BatchParams *runs;
    const SegParams *segs;
    const uint32_t *tile_pref;    // nrun + 1: tile items before run r
    const uint32_t *chk_pref;     // nseg + 1: virtual CTAs of k_check before segment s
    const uint32_t *ver_pref;     // nseg + 1: the same for k_verify
    const uint32_t *cnt_pref;     // nseg + 1: the same for k_count
};

// The next item of a persistent kernel's work counter for the whole CTA
// (every thread gets the same value; the caller's loop body must end with
// a __syncthreads before the next call).
__device__ __forceinline__ uint32_t next_item(uint32_t *counter, uint32_t *s_slot)
{
    if (threadIdx.x == 0) *s_slot = atomicAdd(counter, 1u);
    __syncthreads();
    return *s_slot;
}

// the last index i in [0, n) with pref[i] <= x (pref ascending, pref[0] = 0)
__device__ __forceinline__ uint32_t find_prefix(const uint32_t *pref, uint32_t n, uint32_t x)
{
    uint32_t lo = 0, hi = n;  // pref[lo] <= x < pref[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(pref + mid) <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

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
    const uint2 *fun;       // funnel: candidate index of its smallest member p, members (bit d: p + 30 d, d < 32)
    const uint2 *fpair;     // per funnel: delta, pair starts a (bit a: shifts a and a + delta), or 0, 0
    const uint16_t *rest;   // candidates no funnel tests, ascending
    uint32_t fun_off[GBC_NCLASS], fun_cnt[GBC_NCLASS];
    uint32_t rest_off[GBC_NCLASS], rest_cnt[GBC_NCLASS];
    uint32_t ridge_min;     // evens with p(n) >= ridge_min are listed with their p(n)
    uint32_t f1;            // funnels every word takes before the unresolved ones are gathered (>= 1)
    uint32_t spin0;         // try_wait rounds of the first wait on a chunk's bulk copies (kStageSpin)
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
constexpr uint32_t kErrSelfCheck = 1u << 8;  // the map self-check found differing words
constexpr uint32_t kErrStaging = 1u << 9;    // a bulk copy into shared memory missed its wait limit
constexpr uint32_t kErrHlOverflow = 1u << 10; // more hit-list overflow marks than the overflow list holds

// funnels per class the verify kernel holds (the plan has at most this many)
constexpr uint32_t kVerifyMaxFun = 32;
// shift groups (four shifts each) per funnel: pair starts, then single members
constexpr uint32_t kVerifyMaxGroups = 9;

// tiles per hit-list region k_binsort handles
constexpr uint32_t kSortMaxTiles = 1024;

// ---------------------------------------------------------------------------
// Bulk copies global -> shared memory (cp.async.bulk, the TMA unit's
// untiled form) completing on an mbarrier. Source and destination 16-byte
// aligned, sizes multiples of 16 bytes. Waits are bounded: kStageSpin
// try_wait rounds of at most about a microsecond each.
constexpr uint32_t kStageSpin = 1u << 16;

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes initialised mbarriers visible to the async proxy
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// orders this thread's earlier generic shared-memory accesses (and those it
// synchronised with) before its later async-proxy copies into shared memory
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// the TMA unit's L2 prefetch of a global range (16-byte aligned start, size
// a multiple of 16 bytes); no completion to wait for
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(1000u)
        : "memory");
    return ok != 0;
}

// waits for the phase of the given parity, at most `rounds` try_wait
// rounds; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t rounds = kStageSpin)
{
    for (uint32_t i = 0; i < rounds; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

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

// Host-side launchers (defined in the kernel translation units). Grids are
// fixed per context (persistent kernels looping over the batch's items), so
// the same launches serve every batch and can be captured into a graph.
namespace gbh {
struct Grids {
    int sm = 1;                  // multiprocessors
    int check = 1, verify = 1, count = 1;  // resident CTAs of those kernels
    int hitlist = 1;             // resident CTAs of k_hitlist (its grid: one wave)
    int max_seg = 1;             // segments a batch can hold
};
void launch_init(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st);
void launch_xfirst(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st);
void launch_tile(const gbk::BatchDesc &d, const gbk::GroupInfo &gi, uint32_t tile_bits, uint32_t stage,
                 const Grids &g, cudaStream_t st);
void launch_large(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st);
// direct = false: the binned harvest (before the tiles); true: the direct
// marks of every other batch (after the tiles)
void launch_hitlist(const gbk::BatchDesc &d, bool direct, const Grids &g, cudaStream_t st);
void launch_binsort(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st);
void launch_hl_overflow(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st);
void query_sieve_grids(Grids &g);
void launch_check(const gbk::BatchDesc &d, const gbk::CheckTables &ct, const Grids &g, cudaStream_t st);
void launch_verify(const gbk::BatchDesc &d, const gbk::VerifyTables &vt, const Grids &g, cudaStream_t st);
void launch_retry(const gbk::BatchDesc &d, uint32_t ridge_min, uint32_t tries, const Grids &g, cudaStream_t st);
void launch_count(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st);
void launch_map_compare(const gbk::BatchDesc &a, const gbk::BatchDesc &b, uint32_t *count, const Grids &g,
                        cudaStream_t st);
// the persistent tile kernel's shared memory for tile_bits-bit tiles; sets
// *stage to the tile-bin offsets it can stage (0 when the tile leaves no room)
// and returns false when the tile itself does not fit
bool tile_attributes(uint32_t tile_bits, uint32_t tile_log2, const gbk::GroupInfo &gi, int device, uint32_t *stage);
void query_check_grids(Grids &g);
void query_count_grids(Grids &g);
uint32_t check_vbx(uint64_t evens, int sm);
// single-run forms (the allocation-free entry point and the table build)
void launch_xfirst1(const gbk::BatchParams &bp, cudaStream_t st);
void launch_tile1(const gbk::BatchParams &bp, const gbk::GroupInfo &gi, cudaStream_t st);
void launch_wheel_bytes(const gbk::BatchParams &bp, uint32_t *out, cudaStream_t st);
// host geometry of the count kernel: CountRanges of a segment on its run's map, and its CTAs
uint32_t count_ranges(uint64_t base, const gbk::SegParams &sp, gbk::CountRanges &cr);
}  // namespace gbh
