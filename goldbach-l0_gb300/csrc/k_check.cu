// k_check.cu -- the exact smallest Goldbach prime p(n) of every even.
//
// Evens are grouped by class r = n mod 30 (the reference's check30 layout,
// include/check30.hpp:1-19): for a candidate p, q = n - p of every even of
// class r lies in the class array of residue r - p, and consecutive evens of
// the class are consecutive bits there, so one funnel shift tests 32 evens
// (goldbach.cl:1950-2001). Unlike the reference's phase A (funnels of
// several candidates, any witness), this checker tests the candidates of
// each class in ascending order, so the first candidate that hits an even
// IS p(n): the exact per-even result that the reference only computes on
// sampled segments (check30_xs* + check30_xb, goldbach.cl:2339-2418,
// 2880-3021). Per candidate, a warp reduction adds the hits to the
// histogram and the first occurrence; evens left without a witness <= 9781
// go to a list that k_retry settles on the GPU (the reference's CPU
// fallback cpu_min_goldbach_prime, src/primes.cpp:482-493, moved on device).
//
// Every kernel here is persistent: a fixed grid takes the "virtual CTAs"
// of all segments of the batch (per segment: vbx CTAs per class) from a
// work counter, each found through the batch descriptor's prefix arrays.
#include <cuda_runtime.h>

#include <cstddef>

#include "gbc_common.cuh"

namespace gbk {

__device__ __forceinline__ void append_leftover(gbc_segment_result *res, uint64_t n)
{
    const uint32_t slot = atomicAdd(&res->nleft, 1u);
    if (slot < GBC_LEFT_CAP) res->left_n[slot] = n;
    else atomicOr(&res->err, kErrLeftOverflow);
}

// (n, p(n)) of an even whose smallest witness reaches the ridge floor (the
// reference's ridge appends, include/ridge.hpp:116-165)
__device__ __forceinline__ void append_ridge(gbc_segment_result *res, uint64_t n, uint32_t p)
{
    const uint32_t slot = atomicAdd(&res->nridge, 1u);
    if (slot < GBC_RIDGE_CAP) {
        res->ridge_n[slot] = n;
        res->ridge_p[slot] = p;
    } else atomicOr(&res->err, kErrRidgeOverflow);
}

constexpr int kCheckThreads = 256;
constexpr int kCheckWarps = kCheckThreads / 32;
constexpr uint32_t kWL = 4;                 // words per lane of a warp's chunk
constexpr uint32_t kChunk = 32 * kWL;       // words per chunk
constexpr uint32_t kWin = kChunk + 16;      // staged words per class array per warp: chunk + span of the candidates + 2
constexpr uint32_t kCheckSmem = kCheckWarps * 8 * kWin * 4;  // dynamic shared memory of k_check (bytes)

// valid-even mask of word j of a class with ecount evens
__device__ __forceinline__ uint32_t word_mask(uint32_t j, uint64_t ecount)
{
    const uint64_t e0 = uint64_t(j) * 32;
    if (e0 >= ecount) return 0u;
    return (ecount - e0 >= 32) ? ~0u : ((1u << uint32_t(ecount - e0)) - 1u);
}

__device__ __forceinline__ void write_pn(uint16_t *pn, uint32_t idx0, uint32_t j, uint32_t h, uint16_t pv)
{
    while (h) {
        const uint32_t b = __ffs(h) - 1u;
        pn[idx0 + 15u * (32u * j + b)] = pv;
        h &= h - 1u;
    }
}

// position of the k-th set bit (from 0) of m; m has more than k set bits
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t k)
{
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t s = 16; s > 0; s >>= 1) {
        const uint32_t lo = __popc(m & ((1u << s) - 1u));
        if (k >= lo) {
            k -= lo;
            m >>= s;
            pos += s;
        }
    }
    return pos;
}

// Virtual CTA (chunk column bx of vbx, class r) of a sampled segment; each
// warp takes kChunk consecutive words (32 kWL words, 1024 kWL evens) of class
// r at a time, stages the 8 class-array windows they read (the chunk + the
// candidates' span) in its own shared memory, and tests the class's useful
// candidates in ascending order: lane l holds words l, l + 32, ..., so every
// shared-memory read of the warp is 32 consecutive words. Four words per
// lane share each candidate's warp reduction and bookkeeping among 4096
// evens: against two words per lane, the windows leg's checker took 200.2
// instead of 239.7 ms and p(n) of every even on production segments ran at
// 369 instead of 326 G evens/s (one GB300), although a chunk then waits for
// the slowest of twice as many evens.
__global__ void __launch_bounds__(kCheckThreads) k_check(BatchDesc d, CheckTables ct)
{
    __shared__ uint32_t s_ent[GBC_NCAND];   // word offset | shift << 16
    __shared__ uint16_t s_p[GBC_NCAND];
    __shared__ uint16_t s_ci[GBC_NCAND];
    __shared__ uint32_t s_hist[GBC_NCAND];
    __shared__ uint32_t s_first[GBC_NCAND];
    extern __shared__ __align__(16) uint32_t s_chk_win[];  // kCheckWarps x 8 x kWin words
    __shared__ uint32_t s_dmin, s_dmax, s_cridge;

    __shared__ uint32_t s_vb;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t total = d.h->chk_vb, nseg = d.h->nseg;
    for (;;) {
        const uint32_t vb = next_item(d.work + kWorkCheck, &s_vb);
        if (vb >= total) break;
        const uint32_t si = find_prefix(d.chk_pref, nseg, vb);
        const SegParams &sp = d.segs[si];
        const BatchParams &bp = d.runs[sp.run];
        const uint32_t local = vb - __ldg(d.chk_pref + si);
        const uint32_t cr = local % GBC_NCLASS, bx = local / GBC_NCLASS, gx = sp.vbx, r = 2 * cr;
        const uint64_t seg_start = sp.seg_start, base = bp.base;
        const uint32_t wpc = bp.wpc;
        const uint32_t *map = bp.map;
        gbc_segment_result *res = sp.res;
        uint16_t *pn = sp.pn;
        const uint64_t n0 = seg_start + (r + 30 - uint32_t(seg_start % 30)) % 30;  // first even of class r
        if (n0 > sp.seg_end) {
            __syncthreads();
            continue;
        }
        const uint64_t ecount = (sp.seg_end - n0) / 30 + 1;
        const uint32_t nwords = uint32_t((ecount + 31) / 32);
        const uint32_t ncand = ct.cnt[cr];

        if (tid == 0) {
            s_dmin = kNone;
            s_dmax = 0;
            s_cridge = ncand;  // the first candidate with p >= ridge_min (ascending list)
        }
        __syncthreads();
        // q = n0 + 30 t - p = base + 30 (D + t) + u: D is the bit of the
        // candidate's window at word 0 of class r
        for (uint32_t c = tid; c < ncand; c += blockDim.x) {
            const uint32_t ci = ct.list[ct.off[cr] + c];
            const uint32_t p = ct.cand[ci];
            const uint32_t D = uint32_t((n0 - base - p - (r + 30 - p % 30) % 30) / 30);
            atomicMin(&s_dmin, D);
            atomicMax(&s_dmax, D);
        }
        __syncthreads();
        const uint32_t dlo = s_dmin & ~31u;                        // staged windows start at word dlo / 32 + J
        const uint32_t nstage = (s_dmax - dlo) / 32 + kChunk + 2;  // words per class array (<= kWin)
        for (uint32_t c = tid; c < ncand; c += blockDim.x) {
            const uint32_t ci = ct.list[ct.off[cr] + c];
            const uint32_t p = ct.cand[ci];
            const uint32_t u = (r + 30 - p % 30) % 30;
            const uint32_t dd = uint32_t((n0 - base - p - u) / 30) - dlo;
            // word offset of the window in the warp's staging area | shift << 16
            s_ent[c] = (class_of(u) * kWin + (dd >> 5)) | ((dd & 31) << 16);
            if (p >= ct.ridge_min) atomicMin(&s_cridge, c);
            s_p[c] = uint16_t(p);
            s_ci[c] = uint16_t(ci);
            s_hist[c] = 0;
            s_first[c] = kNone;
        }
        __syncthreads();

        const uint32_t idx0 = uint32_t((n0 - seg_start) / 2);  // index of n0 among the segment's evens
        const uint32_t c_ridge = s_cridge;
        uint32_t *win = s_chk_win + warp * (8 * kWin);
        for (uint32_t ch = bx * kCheckWarps + warp; ch * kChunk < nwords; ch += gx * kCheckWarps) {
            const uint32_t J = ch * kChunk;
            // stage the windows: class array k, words dlo / 32 + J + [0, nstage)
            const uint32_t *src = map + (dlo >> 5) + J;
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k)
                for (uint32_t i = lane; i < nstage; i += 32) win[k * kWin + i] = __ldg(src + size_t(k) * wpc + i);
            __syncwarp();
            uint32_t um[kWL];  // evens of word J + 32 w + lane still without a witness
#pragma unroll
            for (uint32_t w = 0; w < kWL; ++w) um[w] = word_mask(J + 32 * w + lane, ecount);
            const uint32_t chunk_min = idx0 + 15u * 32u * J;  // smallest even index of this chunk
            const uint32_t *wl = win + lane;
            // records the hits h of candidate c (um already updated)
            auto record = [&](uint32_t c, const uint32_t (&h)[kWL], uint32_t cnt) {
                if (s_first[c] > chunk_min) {  // this chunk can still hold the first occurrence
                    uint32_t mine = kNone;
#pragma unroll
                    for (int w = kWL - 1; w >= 0; --w)
                        if (h[w]) mine = idx0 + 15u * (32u * (J + 32u * w + lane) + __ffs(h[w]) - 1u);
                    const uint32_t mn = __reduce_min_sync(~0u, mine);
                    if (lane == 0) atomicMin(&s_first[c], mn);
                }
                if (lane == 0) atomicAdd(&s_hist[c], cnt);
                if (pn) {
#pragma unroll
                    for (uint32_t w = 0; w < kWL; ++w) write_pn(pn, idx0, J + 32 * w + lane, h[w], s_p[c]);
                }
                if (c >= c_ridge) {
#pragma unroll
                    for (uint32_t w = 0; w < kWL; ++w)
                        for (uint32_t x = h[w]; x; x &= x - 1u)
                            append_ridge(res, n0 + 30ull * (32ull * (J + 32 * w + lane) + __ffs(x) - 1u), s_p[c]);
                }
            };
            auto open = [&]() {
                uint32_t o = 0;
#pragma unroll
                for (uint32_t w = 0; w < kWL; ++w) o |= um[w];
                return __any_sync(~0u, o);
            };
            uint32_t c = 0;
            bool gather = false;
            // two candidates per trip: their window reads are independent; the
            // second one only tests what the first one left. Every fourth trip
            // counts the words still open: once they fit one per lane, they
            // are gathered and take the remaining candidates one word per lane
            // (p(n) of every even on 128 production segments: the checker
            // 48.3 -> 46.7 ms)
            for (; c + 1 < ncand; c += 2) {
                if ((c & 7u) == 0) {
                    uint32_t nopen = 0;
#pragma unroll
                    for (uint32_t w = 0; w < kWL; ++w) nopen += __popc(__ballot_sync(~0u, um[w] != 0));
                    if (nopen <= 32) {
                        gather = true;
                        break;
                    }
                }
                const uint32_t e0 = s_ent[c], e1 = s_ent[c + 1];
                const uint32_t *w0 = wl + (e0 & 0xFFFF), *w1 = wl + (e1 & 0xFFFF);
                const uint32_t s0 = e0 >> 16, s1 = e1 >> 16;
                uint32_t h0[kWL], h1[kWL], n0c = 0, n1c = 0;
#pragma unroll
                for (uint32_t w = 0; w < kWL; ++w) {
                    const uint32_t a0 = __funnelshift_r(w0[32 * w], w0[32 * w + 1], s0);
                    const uint32_t a1 = __funnelshift_r(w1[32 * w], w1[32 * w + 1], s1);
                    h0[w] = um[w] & a0;
                    um[w] ^= h0[w];
                    h1[w] = um[w] & a1;
                    um[w] ^= h1[w];
                    n0c += __popc(h0[w]);
                    n1c += __popc(h1[w]);
                }
                // both candidates' hit counts in one reduction (each <= 32 kWL 32 < 2^16)
                const uint32_t cnt = __reduce_add_sync(~0u, n0c + (n1c << 16));
                if (cnt & 0xFFFFu) record(c, h0, cnt & 0xFFFFu);
                if (cnt >> 16) record(c + 1, h1, cnt >> 16);
            }
            if (!gather) {
                // the candidates ran out with more than 32 words open
                if (c < ncand && open()) {
                    const uint32_t e0 = s_ent[c];
                    const uint32_t *w0 = wl + (e0 & 0xFFFF);
                    const uint32_t s0 = e0 >> 16;
                    uint32_t h0[kWL], n0c = 0;
#pragma unroll
                    for (uint32_t w = 0; w < kWL; ++w) {
                        h0[w] = um[w] & __funnelshift_r(w0[32 * w], w0[32 * w + 1], s0);
                        um[w] ^= h0[w];
                        n0c += __popc(h0[w]);
                    }
                    const uint32_t cnt0 = __reduce_add_sync(~0u, n0c);
                    if (cnt0) record(c, h0, cnt0);
                }
#pragma unroll
                for (uint32_t w = 0; w < kWL; ++w)
                    for (uint32_t x = um[w]; x; x &= x - 1u)
                        append_leftover(res, n0 + 30ull * (32ull * (J + 32 * w + lane) + __ffs(x) - 1u));
            } else {
                // lane L takes the L-th open word, in (w, source lane) order
                uint32_t ug = 0, jl = 0, rank = lane;
                bool found = false;
#pragma unroll
                for (uint32_t w = 0; w < kWL; ++w) {
                    const uint32_t b = __ballot_sync(~0u, um[w] != 0);
                    const uint32_t nb = __popc(b);
                    const bool mine = !found && rank < nb;
                    const uint32_t src = mine ? nth_set_bit(b, rank) : lane;
                    const uint32_t v = __shfl_sync(~0u, um[w], src);
                    if (mine) {
                        ug = v;
                        jl = 32 * w + src;
                        found = true;
                    } else if (!found) {
                        rank -= nb;
                    }
                }
                const uint32_t *wg = win + jl;  // the lane's word in the staged windows
                const uint32_t jw = J + jl;     // and in class r
                auto record1 = [&](uint32_t cc, uint32_t h, uint32_t cnt) {
                    if (s_first[cc] > chunk_min) {
                        const uint32_t m1 = h ? idx0 + 15u * (32u * jw + __ffs(h) - 1u) : kNone;
                        const uint32_t mn = __reduce_min_sync(~0u, m1);
                        if (lane == 0) atomicMin(&s_first[cc], mn);
                    }
                    if (lane == 0) atomicAdd(&s_hist[cc], cnt);
                    if (pn) write_pn(pn, idx0, jw, h, s_p[cc]);
                    if (cc >= c_ridge)
                        for (uint32_t x = h; x; x &= x - 1u)
                            append_ridge(res, n0 + 30ull * (32ull * jw + __ffs(x) - 1u), s_p[cc]);
                };
                for (; c < ncand; c += 2) {
                    if (!__any_sync(~0u, ug)) break;
                    const uint32_t e0 = s_ent[c];
                    const uint32_t o0 = e0 & 0xFFFF;
                    const uint32_t h0 = ug & __funnelshift_r(wg[o0], wg[o0 + 1], e0 >> 16);
                    ug ^= h0;
                    uint32_t h1 = 0;
                    if (c + 1 < ncand) {
                        const uint32_t e1 = s_ent[c + 1];
                        const uint32_t o1 = e1 & 0xFFFF;
                        h1 = ug & __funnelshift_r(wg[o1], wg[o1 + 1], e1 >> 16);
                        ug ^= h1;
                    }
                    const uint32_t cnt = __reduce_add_sync(~0u, __popc(h0) + (__popc(h1) << 16));
                    if (cnt & 0xFFFFu) record1(c, h0, cnt & 0xFFFFu);
                    if (cnt >> 16) record1(c + 1, h1, cnt >> 16);
                }
                for (uint32_t x = ug; x; x &= x - 1u)
                    append_leftover(res, n0 + 30ull * (32ull * jw + __ffs(x) - 1u));
            }
            __syncwarp();
        }
        __syncthreads();
        for (uint32_t c = tid; c < ncand; c += blockDim.x) {
            if (s_hist[c]) atomicAdd(&res->hist[cr][s_ci[c]], s_hist[c]);
            if (s_first[c] != kNone) atomicMin(&res->first[s_ci[c]], s_first[c]);
        }
        __syncthreads();
    }
}

// Generic checker for segments that reach q < 7 (seg_start < 9788): one
// thread per even, every candidate ascending, q = 3 and q = 5 prime by
// definition (they are not in the class map), q < 3 ends the search.
__global__ void __launch_bounds__(256) k_check_low(BatchDesc d, const uint16_t *cand, uint32_t ridge_min)
{
    if (!d.h->nlow) return;
    const uint32_t nseg = d.h->nseg;
    for (uint32_t si = d.h->seg0; si < nseg; ++si) {
        const SegParams &sp = d.segs[si];
        if (!sp.low) continue;
        const BatchParams &bp = d.runs[sp.run];
        const uint64_t evens = (sp.seg_end - sp.seg_start) / 2 + 1;
        gbc_segment_result *res = sp.res;
        for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < evens;
             e += uint64_t(gridDim.x) * blockDim.x) {
            const uint64_t n = sp.seg_start + 2 * e;
            const uint32_t cr = uint32_t(n % 30) / 2;
            int ci = -1;
            for (int c = 0; c < GBC_NCAND; ++c) {
                const uint64_t p = cand[c];
                if (p + 3 > n) break;
                const uint64_t q = n - p;
                bool prime;
                if (q == 3 || q == 5) prime = true;
                else if (q % 3 == 0 || q % 5 == 0) prime = false;
                else {
                    const uint64_t t = (q - bp.base) / 30;
                    const uint32_t k = class_of(uint32_t(q % 30));
                    prime = (bp.map[size_t(k) * bp.wpc + (t >> 5)] >> (t & 31)) & 1u;
                }
                if (prime) {
                    ci = c;
                    break;
                }
            }
            if (ci >= 0) {
                atomicAdd(&res->hist[cr][ci], 1u);
                atomicMin(&res->first[ci], uint32_t(e));
                if (sp.pn) sp.pn[e] = cand[ci];
                if (cand[ci] >= ridge_min) append_ridge(res, n, cand[ci]);
            } else {
                append_leftover(res, n);
            }
        }
    }
}

// Evens without a witness <= 9781: ascending odd p > 9781 by Miller-Rabin on
// both p and n - p (n = 4: p = 2). A bounded search of at most max_tries
// candidates: one that runs out sets an error flag instead of looping. A
// CTA per segment.
__global__ void __launch_bounds__(64) k_retry(BatchDesc d, uint32_t ridge_min, uint32_t max_tries)
{
    const uint32_t nseg = d.h->nseg;
    for (uint32_t si = d.h->seg0 + blockIdx.x; si < nseg; si += gridDim.x) {
        const SegParams &sp = d.segs[si];
        gbc_segment_result *res = sp.res;
        const uint32_t nl = res->nleft < GBC_LEFT_CAP ? res->nleft : GBC_LEFT_CAP;
        for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x) {
            const uint64_t n = res->left_n[i];
            uint64_t found = 0;
            if (n == 4) found = 2;
            else {
                uint32_t tries = 0;
                for (uint64_t p = GBC_MAX_CAND + 2; p <= n / 2; p += 2) {
                    if (++tries > max_tries) {
                        atomicOr(&res->err, kErrRetry);
                        break;
                    }
                    if (is_prime_u64_dev(p) && is_prime_u64_dev(n - p)) {
                        found = p;
                        break;
                    }
                }
            }
            res->left_p[i] = found;
            if (sp.pn) sp.pn[(n - sp.seg_start) / 2] = found < 65536 ? uint16_t(found) : 0;
            if (found && found >= ridge_min) append_ridge(res, n, uint32_t(found));
        }
    }
}

constexpr int kVerifyThreads = 128;
constexpr uint32_t kVerifyWarps = kVerifyThreads / 32;
constexpr uint32_t kVW = 6;                // words per lane in a chunk
constexpr uint32_t kVChunk = 32 * kVW;     // words per warp chunk
constexpr uint32_t kVWin = kVChunk + 12;   // staged words per class array and buffer: chunk + funnel span (<= 5) + 3 + alignment (<= 3), a multiple of 4
constexpr uint32_t kMaxFun = kVerifyMaxFun;
constexpr size_t kVerifySmem = size_t(kVerifyWarps) * 2 * 8 * kVWin * 4;  // k_verify's dynamic shared memory

// one chunk's eight class-array windows into a staging buffer: 8 bulk
// copies of `bytes` each, completing on bar (issued by one lane)
__device__ __forceinline__ void stage_chunk(uint32_t *dst, uint64_t *bar, const uint32_t *src, uint32_t wpc,
                                            uint32_t bytes)
{
    mbar_arrive_expect_tx(bar, 8 * bytes);
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k) bulk_copy_g2s(dst + k * kVWin, src + size_t(k) * wpc, bytes, bar);
}

// Funnel entry in shared memory: staged word offset (12 bits) | shift << 12
// | pair groups << 17 | single groups << 21 | delta << 25.
static_assert(7 * kVWin + 7 < 4096, "staged word offsets must fit the funnel entry's 12 bits");
__device__ __forceinline__ uint32_t fent_make(uint32_t off, uint32_t sh, uint32_t nga, uint32_t ngr, uint32_t delta)
{
    return off | (sh << 12) | (nga << 17) | (ngr << 21) | (delta << 25);
}
__device__ __forceinline__ uint32_t fent_off(uint32_t e) { return e & 0xFFFu; }
__device__ __forceinline__ uint32_t fent_sh(uint32_t e) { return (e >> 12) & 31u; }
__device__ __forceinline__ uint32_t fent_nga(uint32_t e) { return (e >> 17) & 15u; }
__device__ __forceinline__ uint32_t fent_ngr(uint32_t e) { return (e >> 21) & 15u; }
__device__ __forceinline__ uint32_t fent_delta(uint32_t e) { return e >> 25; }

// ORs into wa the four shifted windows of one group (a funnel shift uses the
// low 5 bits of its operand)
__device__ __forceinline__ uint32_t group_hits(uint32_t lo, uint32_t hi, uint4 q)
{
    return __funnelshift_r(lo, hi, q.x) | __funnelshift_r(lo, hi, q.y) | __funnelshift_r(lo, hi, q.z) |
           __funnelshift_r(lo, hi, q.w);
}

// The OR over one funnel's members of the 32 candidates' bits of word
// window w (three staged words from w): the top member's 64-bit window at
// bit sh, every other member's the same shifted down by its distance. A
// pair of members a, a + delta is one shift of the window ORed with itself
// shifted by delta (the bits a pair reads stay below 63).
__device__ __forceinline__ uint32_t funnel_hits(const uint32_t *w, uint32_t e, const uint4 *fsh)
{
    const uint32_t x0 = w[0], x1 = w[1], x2 = w[2], sh = fent_sh(e), nga = fent_nga(e), ngr = fent_ngr(e);
    const uint32_t al = __funnelshift_r(x0, x1, sh), ah = __funnelshift_r(x1, x2, sh);
    uint32_t wa = 0;
    if (nga) {
        const uint32_t dl = fent_delta(e);
        const uint32_t bl = al | __funnelshift_r(al, ah, dl), bh = ah | (ah >> dl);
        for (uint32_t g = 0; g < nga; ++g) wa |= group_hits(bl, bh, fsh[g]);
    }
    for (uint32_t g = 0; g < ngr; ++g) wa |= group_hits(al, ah, fsh[nga + g]);
    return wa;
}

// Phase A (the reference's check30_a, kernels/goldbach.cl:2029-2189): any
// witness. Each funnel is a set of plan members p + 30 d (d < 32) of one
// residue class, all prime, whose windows are the same staged words shifted
// by their distance in bits, so one 96-bit read and one funnel shift per
// member test up to 32 candidates for 32 evens. No statistics here: evens
// left without a plan witness go to a pending list of (class, word, bits)
// for k_tail.
//
// Staging: each warp double-buffers its 128-word chunks in shared memory;
// one lane moves the next chunk's eight class-array windows with bulk
// copies (cp.async.bulk on an mbarrier) while the warp tests the current
// one. The windows start 16-byte aligned (the class arrays are, and chunks
// are 128 words apart), o = 0..3 words below the lowest word a funnel reads.
//
// Work balance: every lane holds four words (words l, l + 32, l + 64, l + 96
// of the chunk) through the plan's first f1 funnels, which leave about one
// word in ten with an even still unresolved; the warp then gathers those
// words, one per lane (in rounds of 32), for the plan's other funnels, so
// the last funnels cost one word per lane instead of four and no lane waits
// for the slowest even of 4096.
__global__ void __launch_bounds__(kVerifyThreads, 3) k_verify(BatchDesc d, VerifyTables vt)
{
    __shared__ uint32_t s_fent[kMaxFun];  // see fent_off .. fent_delta
    // per funnel: groups of four window offsets above the top member's, the
    // pair starts first, then the single members, each padded with its first
    __shared__ uint4 s_fsh[kMaxFun][kVerifyMaxGroups];
    // per warp: two staging buffers of eight class-array windows (dynamic
    // shared memory: kVerifySmem bytes)
    extern __shared__ __align__(16) uint32_t s_dyn[];
    uint32_t (*s_win)[2][8 * kVWin] = reinterpret_cast<uint32_t (*)[2][8 * kVWin]>(s_dyn);
    __shared__ __align__(8) uint64_t s_bar[kVerifyWarps][2];
    __shared__ uint32_t s_dmin, s_dmax;
    __shared__ unsigned long long s_pend;

    __shared__ uint32_t s_vb;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint64_t *bar = s_bar[warp];
    if (lane == 0) {
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        mbar_init_fence();
    }
    __syncwarp();
    uint32_t phase = 0;  // bit b: parity of buffer b's next completion
    const uint32_t total = d.h->ver_vb, nseg = d.h->nseg;
    for (;;) {
        const uint32_t vb = next_item(d.work + kWorkVerify, &s_vb);
        if (vb >= total) break;
        const uint32_t si = find_prefix(d.ver_pref, nseg, vb);
        const SegParams &sp = d.segs[si];
        const BatchParams &bp = d.runs[sp.run];
        const uint32_t local = vb - __ldg(d.ver_pref + si);
        const uint32_t cr = local % GBC_NCLASS, bx = local / GBC_NCLASS, gx = sp.vbx, r = 2 * cr;
        const uint64_t seg_start = sp.seg_start, base = bp.base;
        const uint32_t wpc = bp.wpc;
        const uint32_t *map = bp.map;
        const uint64_t n0 = seg_start + (r + 30 - uint32_t(seg_start % 30)) % 30;
        if (n0 > sp.seg_end) {
            __syncthreads();
            continue;
        }
        const uint64_t ecount = (sp.seg_end - n0) / 30 + 1;
        const uint32_t nwords = uint32_t((ecount + 31) / 32);
        const uint32_t nfun = vt.fun_cnt[cr] < kMaxFun ? vt.fun_cnt[cr] : kMaxFun;
        const uint32_t f1 = vt.f1 < nfun ? vt.f1 : nfun;
        gbc_segment_result *res = sp.res;
        uint2 *pend_list = sp.pend;
        const uint32_t pend_cap = sp.pend_cap;

        if (tid == 0) {
            s_dmin = kNone;
            s_dmax = 0;
            s_pend = 0;
        }
        __syncthreads();
        // the lowest window bit of each funnel: its top member p + 30 d
        for (uint32_t f = tid; f < nfun; f += blockDim.x) {
            const uint2 e = vt.fun[vt.fun_off[cr] + f];
            const uint32_t p0 = vt.cand[e.x], dm = 31 - __clz(e.y);
            const uint32_t u = (r + 30 - p0 % 30) % 30;
            const uint32_t dlow = uint32_t((n0 - base - p0 - u) / 30) - dm;
            atomicMin(&s_dmin, dlow);
            atomicMax(&s_dmax, dlow);
        }
        __syncthreads();
        const uint32_t dlo = s_dmin & ~31u, o = (dlo >> 5) & 3u;
        // words each class copy moves: the chunk, the funnels' span and the
        // three words a 96-bit read needs, from the aligned start
        const uint32_t cwords = nfun ? ((s_dmax - dlo) / 32 + kVChunk + 4 + o + 3) & ~3u : 0u;
        if (cwords > kVWin) {  // funnel span beyond the staging buffer: nothing tested
            if (tid == 0) atomicOr(&res->err, kErrStaging);
            __syncthreads();
            continue;
        }
        for (uint32_t f = tid; f < nfun; f += blockDim.x) {
            const uint2 e = vt.fun[vt.fun_off[cr] + f];
            const uint32_t p0 = vt.cand[e.x], dm = 31 - __clz(e.y);
            const uint32_t u = (r + 30 - p0 % 30) % 30;
            const uint32_t dd = uint32_t((n0 - base - p0 - u) / 30) - dm - dlo;
            // member p0 + 30 d's window starts dm - d bits above the top
            // member's (shift space, bit 0: the top member); the host's
            // pairs {a, a + delta} take their members out of the singles
            const uint2 pr = vt.fpair[vt.fun_off[cr] + f];
            const uint32_t S = __brev(e.y) >> (31 - dm), dl = pr.x, A = pr.y;
            const uint32_t R = S & ~(A | (dl ? A << dl : 0u));
            uint32_t ng = 0, nga = 0;
            for (uint32_t sel = 0; sel < 2; ++sel) {
                uint32_t sm = sel ? R : A;
                const uint32_t first = sm ? uint32_t(__ffs(sm) - 1) : 0u;
                while (sm) {
                    uint32_t q[4] = {first, first, first, first};
#pragma unroll
                    for (uint32_t j = 0; j < 4; ++j)
                        if (sm) {
                            q[j] = uint32_t(__ffs(sm) - 1);
                            sm &= sm - 1u;
                        }
                    s_fsh[f][ng++] = make_uint4(q[0], q[1], q[2], q[3]);
                }
                if (!sel) nga = ng;
            }
            s_fent[f] = fent_make(class_of(u) * kVWin + o + (dd >> 5), dd & 31, nga, ng - nga, dl);
        }
        __syncthreads();

        uint32_t pend = 0;
        const uint32_t step = gx * kVerifyWarps;
        if (nfun) {
            const uint32_t bytes = cwords * 4;
            const uint32_t *src0 = map + ((dlo >> 5) - o);
            uint32_t ch = bx * kVerifyWarps + warp, buf = 0;
            if (ch * kVChunk < nwords && lane == 0) {
                fence_proxy_async();
                stage_chunk(s_win[warp][0], bar, src0 + size_t(ch) * kVChunk, wpc, bytes);
            }
            for (; ch * kVChunk < nwords; ch += step, buf ^= 1u) {
                const uint32_t nx = ch + step;
                if (nx * kVChunk < nwords) {
                    __syncwarp();  // every lane is done with the other buffer (the chunk before)
                    if (lane == 0) {
                        fence_proxy_async();
                        stage_chunk(s_win[warp][buf ^ 1u], bar + (buf ^ 1u), src0 + size_t(nx) * kVChunk, wpc, bytes);
                    }
                }
                if (!mbar_wait(bar + buf, (phase >> buf) & 1u, vt.spin0)) {
                    atomicOr(&res->err, kErrStaging);
                    mbar_wait(bar + buf, (phase >> buf) & 1u);
                }
                phase ^= 1u << buf;
                const uint32_t J = ch * kVChunk;
                const uint32_t *win = s_win[warp][buf];
                uint32_t u[kVW];
#pragma unroll
                for (uint32_t w = 0; w < kVW; ++w) u[w] = word_mask(J + lane + 32 * w, ecount);
                // the first f1 funnels on all four words of every lane
                for (uint32_t f = 0; f < f1; ++f) {
                    uint32_t any = 0;
#pragma unroll
                    for (uint32_t w = 0; w < kVW; ++w) any |= u[w];
                    if (!__any_sync(~0u, any)) break;
                    const uint32_t e = s_fent[f];
                    const uint32_t *wl = win + lane + fent_off(e);
                    const uint32_t sh = fent_sh(e), nga = fent_nga(e), ngr = fent_ngr(e), dl = fent_delta(e);
                    uint32_t al[kVW], ah[kVW], wa[kVW];
#pragma unroll
                    for (uint32_t w = 0; w < kVW; ++w) {
                        const uint32_t x0 = wl[32 * w], x1 = wl[32 * w + 1], x2 = wl[32 * w + 2];
                        al[w] = __funnelshift_r(x0, x1, sh);
                        ah[w] = __funnelshift_r(x1, x2, sh);
                        wa[w] = 0;
                    }
                    if (nga) {
                        uint32_t bl[kVW], bh[kVW];
#pragma unroll
                        for (uint32_t w = 0; w < kVW; ++w) {
                            bl[w] = al[w] | __funnelshift_r(al[w], ah[w], dl);
                            bh[w] = ah[w] | (ah[w] >> dl);
                        }
                        for (uint32_t g = 0; g < nga; ++g) {
                            const uint4 q = s_fsh[f][g];
#pragma unroll
                            for (uint32_t w = 0; w < kVW; ++w) wa[w] |= group_hits(bl[w], bh[w], q);
                        }
                    }
                    for (uint32_t g = 0; g < ngr; ++g) {
                        const uint4 q = s_fsh[f][nga + g];
#pragma unroll
                        for (uint32_t w = 0; w < kVW; ++w) wa[w] |= group_hits(al[w], ah[w], q);
                    }
#pragma unroll
                    for (uint32_t w = 0; w < kVW; ++w) u[w] &= ~wa[w];
                }
                // the words still unresolved, gathered one per lane (word
                // order: w-major, then lane) for the other funnels
                uint32_t bal[kVW], cpre[kVW], nun = 0;  // cpre[w]: unresolved words in w' <= w
#pragma unroll
                for (uint32_t w = 0; w < kVW; ++w) {
                    bal[w] = __ballot_sync(~0u, u[w] != 0u);
                    nun += __popc(bal[w]);
                    cpre[w] = nun;
                }
                for (uint32_t r0 = 0; r0 < nun; r0 += 32) {
                    const uint32_t t = r0 + lane;
                    uint32_t wt = 0, before = 0, bm = bal[0];
#pragma unroll
                    for (uint32_t w = 0; w + 1 < kVW; ++w)
                        if (t >= cpre[w]) {
                            wt = w + 1;
                            before = cpre[w];
                            bm = bal[w + 1];
                        }
                    const uint32_t srcl = t < nun ? nth_set_bit(bm, t - before) : 0u;
                    uint32_t uu = 0;
#pragma unroll
                    for (uint32_t w = 0; w < kVW; ++w) {
                        const uint32_t v = __shfl_sync(~0u, u[w], srcl);
                        if (w == wt) uu = v;
                    }
                    if (t >= nun) uu = 0;
                    const uint32_t jl = srcl + 32 * wt;  // the word within the chunk
                    for (uint32_t f = f1; f < nfun; ++f) {
                        if (!__any_sync(~0u, uu)) break;
                        const uint32_t e = s_fent[f];
                        uu &= ~funnel_hits(win + jl + fent_off(e), e, s_fsh[f]);
                    }
                    if (uu) {  // every funnel tried: pending (rare)
                        const uint32_t at = atomicAdd(&res->npend, 1u);
                        if (at < pend_cap) pend_list[at] = make_uint2((cr << 27) | (J + jl), uu);
                        else atomicOr(&res->err, kErrPendOverflow);
                        pend += __popc(uu);
                    }
                }
            }
        } else {
            // no funnels for the class: every word of the warp's chunks is pending
            for (uint32_t ch = bx * kVerifyWarps + warp; ch * kVChunk < nwords; ch += step)
                for (uint32_t jj = ch * kVChunk + lane; jj < ch * kVChunk + kVChunk; jj += 32) {
                    const uint32_t uw = word_mask(jj, ecount);
                    if (!uw) continue;
                    const uint32_t at = atomicAdd(&res->npend, 1u);
                    if (at < pend_cap) pend_list[at] = make_uint2((cr << 27) | jj, uw);
                    else atomicOr(&res->err, kErrPendOverflow);
                    pend += __popc(uw);
                }
        }
        pend = __reduce_add_sync(~0u, pend);
        if (lane == 0 && pend) atomicAdd(&s_pend, (unsigned long long)pend);
        __syncthreads();
        if (tid == 0 && s_pend) atomicAdd((unsigned long long *)&res->pending, s_pend);
        __syncthreads();
    }
}

// Phase B (the reference's check30_b, kernels/goldbach.cl:2210-2306): the
// exact p(n) of every pending even, by the class's rest candidates in
// ascending order (every plan member already failed for it), one thread per
// pending word. The histogram and first occurrences of these evens hold
// every even with p(n) >= the plan bound; ridges above the floor are listed.
// The pending words of all segments of the batch form one index space (a
// prefix over the segments' counts), so the segments' words are settled
// side by side rather than one segment after another.
constexpr int kTailThreads = 256;
static_assert(kTailThreads >= 256, "one thread per segment of a batch for the prefix");

__global__ void __launch_bounds__(kTailThreads) k_tail(BatchDesc d, VerifyTables vt)
{
    __shared__ uint32_t s_pref[2][257];
    const uint32_t nseg = d.h->nseg, tid = threadIdx.x;
    // s_pref[.][s]: pending words of the segments before s (Hillis-Steele)
    {
        uint32_t c = 0;
        if (tid < nseg && tid >= d.h->seg0) {  // the segments of the window
            const SegParams &sp = d.segs[tid];
            const uint32_t np = sp.res->npend;
            c = sp.sampled ? 0u : (np < sp.pend_cap ? np : sp.pend_cap);
        }
        s_pref[0][tid + 1] = c;
        if (tid == 0) s_pref[0][0] = s_pref[1][0] = 0;
        __syncthreads();
        uint32_t src = 0;
        for (uint32_t o = 1; o < 256; o <<= 1, src ^= 1u) {
            uint32_t v = s_pref[src][tid + 1];
            if (tid >= o) v += s_pref[src][tid + 1 - o];
            s_pref[src ^ 1u][tid + 1] = v;
            __syncthreads();
        }
        if (src) {  // the result in s_pref[0]
            s_pref[0][tid + 1] = s_pref[1][tid + 1];
            __syncthreads();
        }
    }
    const uint32_t total = s_pref[0][nseg];
    for (uint32_t g = blockIdx.x * blockDim.x + tid; g < total; g += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nseg;  // s_pref[lo] <= g < s_pref[hi]
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_pref[0][mid] <= g) lo = mid;
            else hi = mid;
        }
        const uint32_t si = lo, i = g - s_pref[0][lo];
        const SegParams &sp = d.segs[si];
        const BatchParams &bp = d.runs[sp.run];
        gbc_segment_result *res = sp.res;
        const uint64_t seg_start = sp.seg_start, base = bp.base;
        {
            const uint2 e = sp.pend[i];
            const uint32_t cr = e.x >> 27, j = e.x & ((1u << 27) - 1), r = 2 * cr;
            uint32_t mask = e.y;
            const uint64_t n0 = seg_start + (r + 30 - uint32_t(seg_start % 30)) % 30;
            const uint32_t idx0 = uint32_t((n0 - seg_start) / 2);
            const uint32_t off = vt.rest_off[cr], cnt = vt.rest_cnt[cr];
            for (uint32_t c = 0; c < cnt && mask; ++c) {
                const uint32_t ci = vt.rest[off + c];
                const uint32_t p = vt.cand[ci];
                const uint32_t u = (r + 30 - p % 30) % 30;
                const uint32_t pos = uint32_t((n0 - base - p - u) / 30) + 32 * j;
                const uint32_t *wk = bp.map + size_t(class_of(u)) * bp.wpc + (pos >> 5);
                const uint32_t hit = mask & __funnelshift_r(__ldg(wk), __ldg(wk + 1), pos & 31);
                if (!hit) continue;
                atomicAdd(&res->hist[cr][ci], uint32_t(__popc(hit)));
                atomicMin(&res->first[ci], idx0 + 15u * (32u * j + __ffs(hit) - 1u));
                if (p >= vt.ridge_min)
                    for (uint32_t h = hit; h; h &= h - 1u)
                        append_ridge(res, n0 + 30ull * (32ull * j + __ffs(h) - 1u), p);
                mask &= ~hit;
            }
            for (; mask; mask &= mask - 1u) append_leftover(res, n0 + 30ull * (32ull * j + __ffs(mask) - 1u));
        }
    }
}

// Result areas of the batch's segments: zero, except the first-occurrence
// indices and the first prime (all ones: none yet); the slot's error word;
// a binned batch's tile-bin and overflow counts.
__global__ void __launch_bounds__(256) k_init(BatchDesc d)
{
    constexpr uint32_t kWords = sizeof(gbc_segment_result) / 4;
    constexpr uint32_t kF0 = offsetof(gbc_segment_result, first) / 4, kF1 = kF0 + GBC_NCAND;
    constexpr uint32_t kP0 = offsetof(gbc_segment_result, first_prime) / 4;
    const uint32_t nseg = d.h->nseg;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid == 0 && d.h->nrun) *d.runs[0].err = 0;
    if (d.h->nrun && hl_binned(d.runs[0])) {  // the tile bins' counts and the overflow count
        const BatchParams &bp = d.runs[0];
        for (uint32_t i = tid; i < 8 * bp.tb_tiles; i += gridDim.x * blockDim.x) bp.tb_cnt[i] = 0;
        if (tid == 0) *bp.ovf_cnt = 0;
    }
    for (uint32_t si = 0; si < nseg; ++si) {
        uint32_t *w = reinterpret_cast<uint32_t *>(d.segs[si].res);
        for (uint32_t i = tid; i < kWords; i += gridDim.x * blockDim.x)
            w[i] = ((i >= kF0 && i < kF1) || i == kP0 || i == kP0 + 1) ? ~0u : 0u;
    }
}

}  // namespace gbk

namespace gbh {

void launch_init(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st)
{
    gbk::k_init<<<g.sm * 2, 256, 0, st>>>(d);
}

// checker CTAs per class of a segment with the given evens (a virtual grid
// column count: each warp about twelve chunks of 128 words, to spread the
// CTA's table setup; at most two per SM). Measured per 128-segment batch
// with every segment sampled, three / six / twelve chunks per warp: 55.4 /
// 50.7 / 48.3 ms.
uint32_t check_vbx(uint64_t evens, int sm)
{
    const uint64_t words = (evens / 15 + 32) / 32 + 1;
    constexpr uint64_t kPerVb = gbk::kCheckWarps * gbk::kChunk * 12;  // about twelve chunks per warp
    uint64_t bx = (words + kPerVb - 1) / kPerVb;
    const uint64_t cap = uint64_t(sm) * 2;
    if (bx > cap) bx = cap;
    if (bx < 1) bx = 1;
    return uint32_t(bx);
}

void launch_check(const gbk::BatchDesc &d, const gbk::CheckTables &ct, const Grids &g, cudaStream_t st)
{
    gbk::k_check_low<<<g.sm * 16, 256, 0, st>>>(d, ct.cand, ct.ridge_min);
    gbk::k_check<<<g.sm * g.check, gbk::kCheckThreads, gbk::kCheckSmem, st>>>(d, ct);
}

void launch_verify(const gbk::BatchDesc &d, const gbk::VerifyTables &vt, const Grids &g, cudaStream_t st)
{
    gbk::k_verify<<<g.sm * g.verify, gbk::kVerifyThreads, gbk::kVerifySmem, st>>>(d, vt);
    gbk::k_tail<<<g.sm * 2, gbk::kTailThreads, 0, st>>>(d, vt);
}

void launch_retry(const gbk::BatchDesc &d, uint32_t ridge_min, uint32_t tries, const Grids &g, cudaStream_t st)
{
    gbk::k_retry<<<g.max_seg < 1024 ? g.max_seg : 1024, 64, 0, st>>>(d, ridge_min, tries);
}

void query_check_grids(Grids &g)
{
    int n = 0;
    cudaFuncSetAttribute(gbk::k_check, cudaFuncAttributeMaxDynamicSharedMemorySize, int(gbk::kCheckSmem));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gbk::k_check, gbk::kCheckThreads, gbk::kCheckSmem);
    g.check = n > 0 ? n : 1;
    n = 0;
    cudaFuncSetAttribute(gbk::k_verify, cudaFuncAttributeMaxDynamicSharedMemorySize, int(gbk::kVerifySmem));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gbk::k_verify, gbk::kVerifyThreads, gbk::kVerifySmem);
    g.verify = n > 0 ? n : 1;
}

}  // namespace gbh
