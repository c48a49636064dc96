// k_count.cu -- per-segment prime, twin and gap statistics and the
// class-map hash, from the finished class map.
//
// The reference's count30 (kernels/goldbach.cl:2571-2825) counts primes per
// residue, three twin types and walks gaps block by block; the host then
// stitches segment boundaries and corrects the run ends
// (include/gstats.hpp:272-296, 533-624, 665-700). Here each segment's map
// reaches 9781 below its first even and 3 above its last one, so every gap
// of a prime counted in the segment has its lower prime inside the map and
// needs no stitching: one thread per 32 blocks of 30 (8 words, one per class
// array); the 8 x 32 bits are transposed to one byte per block so the primes
// come out in natural order; a block-wide sum-scan of the prime counts
// places every thread's primes in one shared list in natural order, whose
// previous entry is each prime's predecessor (a backward word search gives
// the first one's). Positions are 32-bit offsets from the CTA's first block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <initializer_list>

#include "gbc_common.cuh"

namespace gbk {

// bits t in [lo, hi] of word w (t = 32 w + i); hi < lo: empty
__device__ __forceinline__ uint32_t range_mask(uint32_t w, uint32_t lo, uint32_t hi)
{
    if (hi < lo) return 0;
    const uint64_t a0 = uint64_t(w) * 32, a1 = a0 + 31;
    if (hi < a0 || lo > a1) return 0;
    const uint32_t a = lo > a0 ? uint32_t(lo - a0) : 0;
    const uint32_t b = hi < a1 ? uint32_t(hi - a0) : 31;
    return (0xFFFFFFFFu >> (31 - b)) & (0xFFFFFFFFu << a);
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t q)
{
    uint64_t z = q + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// transpose of an 8 x 8 bit matrix: bit 8 i + j -> bit 8 j + i (the
// delta-swap method of Warren, Hacker's Delight, section 7-3)
__device__ __forceinline__ uint64_t transpose8(uint64_t x)
{
    uint64_t t;
    t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
    x = x ^ t ^ (t << 7);
    t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
    x = x ^ t ^ (t << 14);
    t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
    x = x ^ t ^ (t << 28);
    return x;
}

// x - q0 as int32, clamped to +-2^30
__device__ __forceinline__ int32_t rel_clamp(uint64_t x, uint64_t q0)
{
    if (x >= q0) {
        const uint64_t d = x - q0;
        return d > (1u << 30) ? (1 << 30) : int32_t(d);
    }
    const uint64_t d = q0 - x;
    return d > (1u << 30) ? -(1 << 30) : -int32_t(d);
}

// residue of class k (0..7) by one byte permute
__device__ __forceinline__ uint32_t unit_of(uint32_t k) { return __byte_perm(0x0D0B0701u, 0x1D171311u, k) & 0xFF; }

constexpr int kCountThreads = 256;
constexpr int32_t kNoPos = INT32_MIN;
constexpr uint32_t kCountCap = 8192;  // prime positions the CTA's list holds at a time
constexpr uint32_t kCountRounds = 4;  // rounds of kCountThreads words per item (positions stay below 2^20)

// Persistent: a fixed grid takes the virtual CTAs of every segment of the
// batch (per segment: one per 4 x 256 words of its hashed range, taken in
// four rounds of 256) from a work counter. Six CTAs per SM (the most the
// 37 KB of shared memory allows; 40 registers and a few spills): 6.72 ms
// per 128-segment batch against 6.97 at five and 7.24 at four.
__global__ void __launch_bounds__(kCountThreads, 6) k_count(BatchDesc d)
{
    __shared__ uint32_t s_ghist[GBC_GBINS];
    __shared__ uint32_t s_wsum[kCountThreads / 32];
    __shared__ int32_t s_pos[kCountCap];
    __shared__ int32_t s_prev0;
    __shared__ uint32_t s_cnt[8 + 3 + 1];
    __shared__ uint32_t s_key;
    __shared__ int32_t s_first, s_last;
    __shared__ unsigned long long s_hash;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ uint32_t s_vb;
    const uint32_t total = d.h->cnt_vb, nseg = d.h->nseg;
    for (;;) {
        const uint32_t vb = next_item(d.work + kWorkCount, &s_vb);
        if (vb >= total) break;
        const uint32_t si = find_prefix(d.cnt_pref, nseg, vb);
        const SegParams &sp = d.segs[si];
        const BatchParams &bp = d.runs[sp.run];
        const CountRanges &cr = sp.cr;
        const uint32_t vbx = vb - __ldg(d.cnt_pref + si);
        for (uint32_t i = tid; i < GBC_GBINS; i += blockDim.x) s_ghist[i] = 0;
        if (tid < 12) s_cnt[tid] = 0;
        const uint32_t wi0 = cr.w_lo + vbx * kCountThreads * kCountRounds;  // first word of the item
        const uint64_t q0 = bp.base + 30ull * 32ull * wi0;                   // q of relative position 0
        if (tid == 0) {
            s_key = 0;
            s_first = INT32_MAX;
            s_last = kNoPos;
            s_hash = 0;
            // last hashed prime before the item's first word (negative position)
            int32_t pv = kNoPos;
            for (int64_t ww = int64_t(wi0) - 1; ww >= int64_t(cr.w_lo) && pv == kNoPos; --ww) {
                for (uint32_t k = 0; k < 8; ++k) {
                    const uint32_t v = bp.map[size_t(k) * bp.wpc + ww] &
                                       range_mask(uint32_t(ww), cr.hash_t[k][0], cr.hash_t[k][1]);
                    if (v) {
                        const int32_t pos =
                            int32_t(30 * (32 * (ww - int64_t(wi0)) + 31 - __clz(v))) + int32_t(unit_of(k));
                        if (pos > pv) pv = pos;
                    }
                }
            }
            s_prev0 = pv;
        }
        // the counted range as positions relative to q0 (the item's positions
        // stay below 2^20, so clamping at +-2^30 changes nothing)
        const int32_t clo = rel_clamp(sp.cnt_lo, q0), chi = rel_clamp(sp.cnt_hi, q0);
        const bool hash = !(sp.flags & GBC_SEG_NOHASH);
        uint64_t hsum = 0;
        uint32_t key = 0, err = 0, nh_all = 0, tw[3] = {0u, 0u, 0u}, cc[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        int32_t cfirst = INT32_MAX, clast = kNoPos;
        int32_t carry = kNoPos;  // the prime before the current list's first entry

        for (uint32_t rd = 0; rd < kCountRounds; ++rd) {
            const uint32_t wr0 = wi0 + rd * kCountThreads;  // first word of the round
            if (wr0 > cr.w_hi) break;
            const uint32_t w = wr0 + tid;
            const bool valid = w <= cr.w_hi;
            const bool inner = w >= cr.in_lo && w <= cr.in_hi;
            uint32_t h[8], raw[8];
    #pragma unroll
            for (uint32_t k = 0; k < 8; ++k) {
                raw[k] = valid ? bp.map[size_t(k) * bp.wpc + w] : 0u;
                h[k] = inner ? raw[k] : raw[k] & range_mask(w, cr.hash_t[k][0], cr.hash_t[k][1]);
                cc[k] += __popc(inner ? raw[k] : raw[k] & range_mask(w, cr.cnt_t[k][0], cr.cnt_t[k][1]));
            }
            // twins (11, 13), (17, 19) inside a block; (29, 31) into the next block
            const uint32_t next0 = valid ? bp.map[w + 1] : 0u;  // class 0, word w + 1
            const uint32_t up29 = (raw[0] >> 1) | (next0 << 31);
            tw[0] += __popc(raw[2] & raw[3] & (inner ? ~0u : range_mask(w, cr.twin_t[2][0], cr.twin_t[2][1])));
            tw[1] += __popc(raw[4] & raw[5] & (inner ? ~0u : range_mask(w, cr.twin_t[4][0], cr.twin_t[4][1])));
            tw[2] += __popc(raw[7] & up29 & (inner ? ~0u : range_mask(w, cr.twin_t[7][0], cr.twin_t[7][1])));

            // one byte per block, natural order: word i of T holds blocks 4 i .. 4 i + 3
            uint32_t T[8];
    #pragma unroll
            for (uint32_t g = 0; g < 4; ++g) {
                const uint32_t sel = g | ((g + 4) << 4);
                const uint32_t lo = __byte_perm(__byte_perm(h[0], h[1], sel), __byte_perm(h[2], h[3], sel), 0x5410);
                const uint32_t hi = __byte_perm(__byte_perm(h[4], h[5], sel), __byte_perm(h[6], h[7], sel), 0x5410);
                const uint64_t t = transpose8((uint64_t(hi) << 32) | lo);
                T[2 * g] = uint32_t(t);
                T[2 * g + 1] = uint32_t(t >> 32);
            }
            const int32_t cbase = int32_t(960 * (rd * kCountThreads + tid));  // this thread's first block
            uint32_t nh = 0;
    #pragma unroll
            for (int i = 0; i < 8; ++i) nh += __popc(T[i]);
            nh_all += nh;
            // exclusive sum-scan of the prime counts over the CTA: this thread's
            // primes are entries [off, off + nh) of the round's list in natural order
            uint32_t v = nh;
    #pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t n = __shfl_up_sync(~0u, v, o);
                if (lane >= uint32_t(o)) v += n;
            }
            if (lane == 31) s_wsum[warp] = v;
            __syncthreads();
            if (rd == 0) carry = s_prev0;
            uint32_t off = v - nh, ntot = 0;
            for (uint32_t i = 0; i < kCountThreads / 32; ++i) {
                const uint32_t sw = s_wsum[i];
                if (i < warp) off += sw;
                ntot += sw;
            }

            // the primes in natural order, kCountCap at a time: each thread
            // writes its own into the list (phase 1), then the CTA takes the
            // list in stride (phase 2: the hash of all, the gaps of the
            // counted ones), so the per-prime work has no divergence between
            // lanes
            for (uint32_t lo = 0; lo < ntot; lo += kCountCap) {
                const uint32_t n = ntot - lo < kCountCap ? ntot - lo : kCountCap;
                if (off < lo + n && off + nh > lo) {
                    uint32_t idx = off - lo;  // wraps below the list: skipped by idx < n
    #pragma unroll
                    for (uint32_t i = 0; i < 8; ++i) {
                        uint32_t x = T[i];
                        while (x) {
                            const uint32_t b = __ffs(x) - 1u;
                            x &= x - 1u;
                            if (idx < n) s_pos[idx] = cbase + int32_t(30 * (4 * i + (b >> 3)) + unit_of(b & 7));
                            ++idx;
                        }
                    }
                }
                __syncthreads();
                for (uint32_t k = tid; k < n; k += kCountThreads) {
                    const int32_t pos = s_pos[k];
                    const int32_t prev = k ? s_pos[k - 1] : carry;
                    if (hash) hsum += splitmix64(q0 + uint64_t(int64_t(pos)));
                    if (pos >= clo && pos <= chi) {
                        if (pos < cfirst) cfirst = pos;
                        if (pos > clast) clast = pos;
                        if (prev != kNoPos) {
                            const uint32_t g = uint32_t(pos - prev);
                            if (g / 2 >= GBC_GBINS) err |= kErrGapRange;
                            else atomicAdd(&s_ghist[g / 2], 1u);
                            // largest gap, the smallest lower prime on ties: g << 21 | ~(lower + 2^20)
                            const uint32_t k2 = (g << 21) | (0x1FFFFFu - uint32_t(prev + (1 << 20)));
                            if (k2 > key) key = k2;
                            if (g >= GBC_GTAIL) {
                                const uint32_t slot = atomicAdd(&sp.res->ntail, 1u);
                                if (slot < GBC_TAIL_CAP) {
                                    sp.res->tail_g[slot] = g;
                                    sp.res->tail_lo[slot] = q0 + uint64_t(int64_t(prev));
                                } else err |= kErrTailOverflow;
                            }
                        } else if (q0 + uint64_t(int64_t(pos)) > 7) {
                            err |= kErrNoPred;
                        }
                    }
                }
                carry = s_pos[n - 1];
                __syncthreads();  // the list is rewritten next
            }
        }
        if (err) atomicOr(&sp.res->err, err);

        // warp reductions, then one shared atomic per warp
    #pragma unroll
        for (int o = 16; o > 0; o >>= 1) hsum += __shfl_xor_sync(~0u, hsum, o);
        key = __reduce_max_sync(~0u, key);
        cfirst = __reduce_min_sync(~0u, cfirst);
        clast = __reduce_max_sync(~0u, clast);
        uint32_t r8[12];
    #pragma unroll
        for (int k = 0; k < 8; ++k) r8[k] = __reduce_add_sync(~0u, cc[k]);
        r8[8] = __reduce_add_sync(~0u, tw[0]);
        r8[9] = __reduce_add_sync(~0u, tw[1]);
        r8[10] = __reduce_add_sync(~0u, tw[2]);
        r8[11] = __reduce_add_sync(~0u, nh_all);
        if (lane == 0) {
    #pragma unroll
            for (int k = 0; k < 12; ++k) atomicAdd(&s_cnt[k], r8[k]);
            atomicAdd(&s_hash, (unsigned long long)hsum);
            atomicMax(&s_key, key);
            atomicMin(&s_first, cfirst);
            atomicMax(&s_last, clast);
        }
        __syncthreads();
        gbc_segment_result *res = sp.res;
        for (uint32_t i = tid; i < GBC_GBINS; i += blockDim.x)
            if (s_ghist[i]) atomicAdd(&res->ghist[i], s_ghist[i]);
        if (tid < 8) {
            if (s_cnt[tid]) atomicAdd((unsigned long long *)&res->primes30[tid], (unsigned long long)s_cnt[tid]);
        } else if (tid < 11) {
            if (s_cnt[tid]) atomicAdd((unsigned long long *)&res->twins[tid - 8], (unsigned long long)s_cnt[tid]);
        } else if (tid == 11) {
            if (hash) atomicAdd((unsigned long long *)&res->map_hash, s_hash);
            atomicAdd((unsigned long long *)&res->map_primes, (unsigned long long)s_cnt[11]);
        } else if (tid == 12) {
            if (s_key) {
                const uint64_t g = s_key >> 21;
                const uint64_t lower = q0 + uint64_t(int64_t(int32_t(0x1FFFFFu - (s_key & 0x1FFFFFu)) - (1 << 20)));
                const unsigned long long k64 = (g << 32) | (0xFFFFFFFFull - uint32_t(lower - sp.hash_lo));
                atomicMax((unsigned long long *)&res->gmax_key, k64);
            }
        } else if (tid == 13) {
            if (s_first != INT32_MAX)
                atomicMin((unsigned long long *)&res->first_prime, (unsigned long long)(q0 + uint64_t(int64_t(s_first))));
            if (s_last != kNoPos)
                atomicMax((unsigned long long *)&res->last_prime, (unsigned long long)(q0 + uint64_t(int64_t(s_last))));
        }
        __syncthreads();
    }
}

}  // namespace gbk

namespace gbh {

// per class k: the bits t of q = base + 30 t + u_k in [a, b]
static void class_range(uint64_t base, uint64_t a, uint64_t b, uint32_t out[8][2])
{
    for (uint32_t k = 0; k < 8; ++k) {
        const uint64_t u = gbk::unit30(k);
        uint64_t lo, hi;
        if (b < base + u || b < a) {
            out[k][0] = 1;
            out[k][1] = 0;
            continue;
        }
        lo = a <= base + u ? 0 : (a - base - u + 29) / 30;
        hi = (b - base - u) / 30;
        if (hi < lo) {
            out[k][0] = 1;
            out[k][1] = 0;
            continue;
        }
        out[k][0] = uint32_t(lo);
        out[k][1] = uint32_t(hi);
    }
}

// words [lo, hi] fully inside the bit ranges of every class (hi < lo: none)
static void inner_words(const uint32_t t[8][2], uint32_t &lo, uint32_t &hi)
{
    uint64_t l = 0, h = UINT32_MAX;
    for (int k = 0; k < 8; ++k) {
        if (t[k][1] < t[k][0]) {
            lo = 1;
            hi = 0;
            return;
        }
        l = std::max<uint64_t>(l, (uint64_t(t[k][0]) + 31) / 32);
        const uint64_t e = (uint64_t(t[k][1]) + 1) / 32;  // first word not entirely inside
        h = std::min<uint64_t>(h, e == 0 ? 0 : e - 1);
        if (e == 0) {
            lo = 1;
            hi = 0;
            return;
        }
    }
    lo = uint32_t(l);
    hi = uint32_t(h);
}

uint32_t count_ranges(uint64_t base, const gbk::SegParams &sp, gbk::CountRanges &cr)
{
    class_range(base, sp.hash_lo, sp.hash_hi, cr.hash_t);
    class_range(base, sp.cnt_lo, sp.cnt_hi, cr.cnt_t);
    class_range(base, sp.cnt_lo, sp.twin_hi, cr.twin_t);
    uint32_t tlo = 0xFFFFFFFFu, thi = 0;
    for (int k = 0; k < 8; ++k)
        if (cr.hash_t[k][1] >= cr.hash_t[k][0]) {
            if (cr.hash_t[k][0] < tlo) tlo = cr.hash_t[k][0];
            if (cr.hash_t[k][1] > thi) thi = cr.hash_t[k][1];
        }
    if (tlo > thi) {
        cr.w_lo = 1;
        cr.w_hi = 0;
        cr.in_lo = 1;
        cr.in_hi = 0;
        return 0;
    }
    cr.w_lo = tlo / 32;
    cr.w_hi = thi / 32;
    uint32_t a0, a1, b0, b1, c0, c1;
    inner_words(cr.hash_t, a0, a1);
    inner_words(cr.cnt_t, b0, b1);
    inner_words(cr.twin_t, c0, c1);
    cr.in_lo = std::max({a0, b0, c0});
    cr.in_hi = std::min({a1, b1, c1});
    const uint32_t nw = cr.w_hi - cr.w_lo + 1;
    constexpr uint32_t kPerItem = gbk::kCountThreads * gbk::kCountRounds;
    return (nw + kPerItem - 1) / kPerItem;
}

void launch_count(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st)
{
    gbk::k_count<<<g.sm * g.count, gbk::kCountThreads, 0, st>>>(d);
}

void query_count_grids(Grids &g)
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gbk::k_count, gbk::kCountThreads, 0);
    g.count = n > 0 ? n : 1;
}

}  // namespace gbh
