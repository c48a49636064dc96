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
// array), primes visited in natural order, a block-wide max-scan of the
// last prime position to give each thread its predecessor, a backward word
// search for the first thread of a CTA.
#include <cuda_runtime.h>

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

struct CountRanges {
    uint32_t hash_t[8][2];  // per class: bits of the hashed q range (inclusive)
    uint32_t cnt_t[8][2];   // bits of the counted primes
    uint32_t twin_t[8][2];  // bits of the counted lower twin primes
    uint32_t w_lo, w_hi;    // words covering the hashed range
};

constexpr int kCountThreads = 256;

__global__ void __launch_bounds__(kCountThreads) k_count(BatchParams bp, SegParams sp, CountRanges cr)
{
    __shared__ uint32_t s_ghist[GBC_GBINS];
    __shared__ unsigned long long s_gmax, s_hash, s_first, s_last, s_prev0, s_nprime;
    __shared__ unsigned long long s_wlast[kCountThreads / 32];
    __shared__ uint32_t s_cnt[8 + 3];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (uint32_t i = tid; i < GBC_GBINS; i += blockDim.x) s_ghist[i] = 0;
    if (tid < 11) s_cnt[tid] = 0;
    const uint32_t wc0 = cr.w_lo + blockIdx.x * blockDim.x;  // first word of the CTA
    if (tid == 0) {
        s_gmax = 0;
        s_hash = 0;
        s_nprime = 0;
        s_first = ~0ull;
        s_last = 0;
        // last hashed prime before the CTA's first word (pos + 1; 0 = none)
        unsigned long long pv = 0;
        for (int64_t ww = int64_t(wc0) - 1; ww >= int64_t(cr.w_lo) && !pv; --ww) {
            for (uint32_t k = 0; k < 8; ++k) {
                const uint32_t v = bp.map[size_t(k) * bp.wpc + ww] &
                                   range_mask(uint32_t(ww), cr.hash_t[k][0], cr.hash_t[k][1]);
                if (v) {
                    const uint64_t pos = 30ull * (32ull * uint64_t(ww) + 31 - __clz(v)) + unit30(k);
                    if (pos + 1 > pv) pv = pos + 1;
                }
            }
        }
        s_prev0 = pv;
    }
    const uint32_t w = wc0 + tid;
    const bool valid = w <= cr.w_hi;
    uint32_t h[8], c[8], raw[8];
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k) {
        raw[k] = valid ? bp.map[size_t(k) * bp.wpc + w] : 0u;
        h[k] = raw[k] & range_mask(w, cr.hash_t[k][0], cr.hash_t[k][1]);
        c[k] = raw[k] & range_mask(w, cr.cnt_t[k][0], cr.cnt_t[k][1]);
    }
    // twins (11, 13), (17, 19) inside a block; (29, 31) into the next block
    const uint32_t next0 = valid ? bp.map[w + 1] : 0u;  // class 0, word w + 1
    const uint32_t up29 = (raw[0] >> 1) | (next0 << 31);
    const uint32_t tw0 = __popc(raw[2] & raw[3] & range_mask(w, cr.twin_t[2][0], cr.twin_t[2][1]));
    const uint32_t tw1 = __popc(raw[4] & raw[5] & range_mask(w, cr.twin_t[4][0], cr.twin_t[4][1]));
    const uint32_t tw2 = __popc(raw[7] & up29 & range_mask(w, cr.twin_t[7][0], cr.twin_t[7][1]));

    // first / last hashed prime of this thread's chunk (pos + 1; 0 = none)
    unsigned long long mylast = 0;
    uint64_t hsum = 0;
    uint32_t nh = 0;
    uint32_t occ = 0;
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k) {
        occ |= h[k];
        nh += __popc(h[k]);
        if (h[k]) {
            const uint64_t pl = 30ull * (32ull * w + 31 - __clz(h[k])) + unit30(k) + 1;
            if (pl > mylast) mylast = pl;
        }
        uint32_t v = (sp.flags & GBC_SEG_NOHASH) ? 0u : h[k];
        while (v) {
            const uint32_t b = __ffs(v) - 1u;
            hsum += splitmix64(bp.base + 30ull * (32ull * w + b) + unit30(k));
            v &= v - 1u;
        }
    }
    // exclusive max-scan of mylast over the CTA
    unsigned long long v = mylast;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long n = __shfl_up_sync(~0u, v, o);
        if (lane >= uint32_t(o) && n > v) v = n;
    }
    unsigned long long excl = __shfl_up_sync(~0u, v, 1);
    if (lane == 0) excl = 0;
    if (lane == 31) s_wlast[warp] = v;
    __syncthreads();
    unsigned long long prev = s_prev0;
    if (excl > prev) prev = excl;
    for (uint32_t i = 0; i < warp; ++i)
        if (s_wlast[i] > prev) prev = s_wlast[i];

    // gaps of the counted primes, in natural order
    unsigned long long gmax = 0, cfirst = ~0ull, clast = 0;
    uint32_t err = 0;
    while (occ) {
        const uint32_t b = __ffs(occ) - 1u;
        occ &= occ - 1u;
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) {
            if (!((h[k] >> b) & 1u)) continue;
            const uint64_t pos = 30ull * (32ull * w + b) + unit30(k);
            if ((c[k] >> b) & 1u) {
                const uint64_t q = bp.base + pos;
                if (q < cfirst) cfirst = q;
                if (q > clast) clast = q;
                if (prev) {
                    const uint64_t g = pos + 1 - prev;
                    const uint64_t lower = q - g;
                    if (g / 2 >= GBC_GBINS) err |= kErrGapRange;
                    else atomicAdd(&s_ghist[g / 2], 1u);
                    const unsigned long long key =
                        (g << 32) | (0xFFFFFFFFull - uint32_t(lower - sp.hash_lo));
                    if (key > gmax) gmax = key;
                    if (g >= GBC_GTAIL) {
                        const uint32_t slot = atomicAdd(&sp.res->ntail, 1u);
                        if (slot < GBC_TAIL_CAP) {
                            sp.res->tail_g[slot] = uint32_t(g);
                            sp.res->tail_lo[slot] = lower;
                        } else err |= kErrTailOverflow;
                    }
                } else if (q > 7) {
                    err |= kErrNoPred;
                }
            }
            prev = pos + 1;
        }
    }
    if (err) atomicOr(&sp.res->err, err);

    // warp reductions of the 64-bit values first (shared 64-bit min / max /
    // add contended by a whole CTA would serialize), then one atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long hs = __shfl_xor_sync(~0u, hsum, o);
        const unsigned long long gm = __shfl_xor_sync(~0u, gmax, o);
        const unsigned long long cf = __shfl_xor_sync(~0u, cfirst, o);
        const unsigned long long cl = __shfl_xor_sync(~0u, clast, o);
        hsum += hs;
        if (gm > gmax) gmax = gm;
        if (cf < cfirst) cfirst = cf;
        if (cl > clast) clast = cl;
    }

    // block reductions
    const uint32_t r0 = __reduce_add_sync(~0u, __popc(c[0])), r1 = __reduce_add_sync(~0u, __popc(c[1]));
    const uint32_t r2 = __reduce_add_sync(~0u, __popc(c[2])), r3 = __reduce_add_sync(~0u, __popc(c[3]));
    const uint32_t r4 = __reduce_add_sync(~0u, __popc(c[4])), r5 = __reduce_add_sync(~0u, __popc(c[5]));
    const uint32_t r6 = __reduce_add_sync(~0u, __popc(c[6])), r7 = __reduce_add_sync(~0u, __popc(c[7]));
    const uint32_t t0 = __reduce_add_sync(~0u, tw0), t1 = __reduce_add_sync(~0u, tw1);
    const uint32_t t2 = __reduce_add_sync(~0u, tw2), nhs = __reduce_add_sync(~0u, nh);
    if (lane == 0) {
        atomicAdd(&s_cnt[0], r0);
        atomicAdd(&s_cnt[1], r1);
        atomicAdd(&s_cnt[2], r2);
        atomicAdd(&s_cnt[3], r3);
        atomicAdd(&s_cnt[4], r4);
        atomicAdd(&s_cnt[5], r5);
        atomicAdd(&s_cnt[6], r6);
        atomicAdd(&s_cnt[7], r7);
        atomicAdd(&s_cnt[8], t0);
        atomicAdd(&s_cnt[9], t1);
        atomicAdd(&s_cnt[10], t2);
        atomicAdd(&s_nprime, (unsigned long long)nhs);
        atomicAdd(&s_hash, (unsigned long long)hsum);
        if (gmax) atomicMax(&s_gmax, gmax);
        if (cfirst != ~0ull) atomicMin(&s_first, cfirst);
        if (clast) atomicMax(&s_last, clast);
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
        atomicAdd((unsigned long long *)&res->map_hash, s_hash);
        atomicAdd((unsigned long long *)&res->map_primes, s_nprime);
    } else if (tid == 12) {
        if (s_gmax) atomicMax((unsigned long long *)&res->gmax_key, s_gmax);
    } else if (tid == 13) {
        if (s_first != ~0ull) atomicMin((unsigned long long *)&res->first_prime, s_first);
        if (s_last) atomicMax((unsigned long long *)&res->last_prime, s_last);
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

void launch_count(const gbk::BatchParams &bp, const gbk::SegParams &sp, cudaStream_t st)
{
    gbk::CountRanges cr;
    class_range(bp.base, sp.hash_lo, sp.hash_hi, cr.hash_t);
    class_range(bp.base, sp.cnt_lo, sp.cnt_hi, cr.cnt_t);
    class_range(bp.base, sp.cnt_lo, sp.twin_hi, cr.twin_t);
    uint32_t tlo = 0xFFFFFFFFu, thi = 0;
    for (int k = 0; k < 8; ++k)
        if (cr.hash_t[k][1] >= cr.hash_t[k][0]) {
            if (cr.hash_t[k][0] < tlo) tlo = cr.hash_t[k][0];
            if (cr.hash_t[k][1] > thi) thi = cr.hash_t[k][1];
        }
    if (tlo > thi) return;
    cr.w_lo = tlo / 32;
    cr.w_hi = thi / 32;
    const uint32_t nw = cr.w_hi - cr.w_lo + 1;
    const uint32_t blocks = (nw + gbk::kCountThreads - 1) / gbk::kCountThreads;
    gbk::k_count<<<blocks, gbk::kCountThreads, 0, st>>>(bp, sp, cr);
}

}  // namespace gbh
