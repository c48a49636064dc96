// k_sieve.cu -- builds the mod-30 class maps of a batch on the GPU.
//
// Stages (the reference's make_prime_map, mid_setup/mid_window and
// sieve_large_packed, kernels/goldbach.cl:1092-1608, 3528-3701, 1738-1849,
// re-designed for HBM-resident maps, one per run of consecutive segments,
// and persistent kernels that take every run of the batch in one launch):
//   k_xfirst  per tile-sieve prime, class and run: the first class bit of
//             the run that is a multiple of p and >= p^2 (mid_setup's job,
//             goldbach.cl:3528-3563; host_math.cpp:80-113).
//   k_tile    one CTA per (run, class, tile) item: up to 2^tile_log2 bits in
//             shared memory; the primes 7..67 by whole-word AND patterns of
//             seven prime groups, then every prime 71..p_mid by shared-memory
//             atomics (small primes warp-cooperatively, the rest one per
//             thread); one coalesced store of the finished tile.
//   k_large   primes in (p_mid, p_hl), streamed at one byte per prime and
//             decoded by warps, every run they reach: every multiple p m (m
//             coprime to 30) by a global atomic AND after a read
//             (read-before-mark, goldbach.cl:328-336), stepping over the
//             multipliers with a factor 7..43, whose multiples the pattern
//             stage clears (the 30030 wheel and the 17..43 skip of
//             goldbach.cl:638-748).
//   k_hitlist the primes above p_hl through the prime-multiplier table.
// A thread reads its prime once and applies it to every run of the batch,
// so a batch of many short windows streams the sieving primes once.
#include <cuda_runtime.h>

#include <algorithm>

#include "gbc_common.cuh"

namespace gbk {

// x mod p, exactly, for x < p * 2^32 and 3 <= p < 2^32, without a
// division: a float estimate of the quotient (error below 2^11 for these
// bounds), an exact 64-bit remainder r (negative when the estimate was
// high), a second float estimate of the now small quotient r / p (error
// below 1), and a final +-p correction. rp = 1/p rounded to nearest.
__device__ __forceinline__ uint32_t mod_below(uint64_t x, uint32_t p, float rp)
{
    // float(x) from its two 32-bit halves (32-bit conversions only: 64-bit
    // integer <-> float conversions are multi-instruction sequences)
    const float xf = fmaf(__uint2float_rz(uint32_t(x >> 32)), 4294967296.0f, __uint2float_rz(uint32_t(x)));
    const uint32_t qe = __float2uint_rz(xf * rp);
    int64_t r = int64_t(x - uint64_t(qe) * p);
    // |r| < 2^43: float(|r|) from its halves as above, then the sign (the
    // halves of a negative r would lose up to 2^8 in the low word's
    // conversion, too much for p below 2^9)
    const uint64_t m = r < 0 ? uint64_t(-r) : uint64_t(r);
    const float mf = fmaf(__uint2float_rz(uint32_t(m >> 32)), 4294967296.0f, __uint2float_rz(uint32_t(m)));
    const float rf = r < 0 ? -mf : mf;
    const int32_t q2 = __float2int_rn(rf * rp);
    r -= int64_t(q2) * p;
    if (r < 0) r += p;
    if (r >= int64_t(p)) r -= p;
    return uint32_t(r);
}

// x mod p for any 64-bit x (two base-2^32 digits)
__device__ __forceinline__ uint32_t mod_u64(uint64_t x, uint32_t p, float rp)
{
    const uint32_t hi = uint32_t(x >> 32);
    const uint32_t r = hi < p ? hi : mod_below(hi, p, rp);
    return mod_below((uint64_t(r) << 32) | uint32_t(x), p, rp);
}

// a + d mod p for a, d < p without overflow
__device__ __forceinline__ uint32_t addmod(uint32_t a, uint32_t d, uint32_t p)
{
    return a >= p - d ? a - (p - d) : a + d;
}

// First class bit, for each class k, of a multiple of p in the run with
// q >= p^2; kNone when the first one is at or past nblk. 29 < p < 2^31.
__device__ __forceinline__ void first_bits8(uint64_t base, uint32_t nblk, uint32_t p, uint32_t *out)
{
    const float rp = __frcp_rn(float(p));
    const uint32_t r = mod_u64(base, p, rp);
    const uint32_t iv = inv30_mod(p);
    const uint64_t pp = uint64_t(p) * p;
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k) {
        const uint32_t u = unit30(k);
        uint32_t a = r + u;                                  // (base + u) mod p
        if (a >= p) a -= p;
        a = a ? p - a : 0;                                   // -(base + u) mod p
        uint64_t t = mod_below(uint64_t(a) * iv, p, rp);     // base + 30 t + u = 0 (mod p)
        const uint64_t q = base + 30 * t + u;
        if (q < pp) {                                        // p itself and smaller multiples stay unmarked
            const uint64_t tmin = (pp - base - u + 29) / 30;
            if (tmin > t) t += (tmin - t + p - 1) / p * p;
        }
        out[k] = t < nblk ? uint32_t(t) : kNone;
    }
}

// every run's first bits of the tile-sieve primes
__global__ void __launch_bounds__(256) k_xfirst(BatchDesc d)
{
    const uint32_t nrun = d.h->nrun, nmax = d.h->n_mid_max;
    if (!nrun) return;
    const uint32_t *primes = d.runs[0].primes;
    for (uint32_t i = d.runs[0].i0 + blockIdx.x * blockDim.x + threadIdx.x; i < nmax; i += gridDim.x * blockDim.x) {
        const uint32_t p = primes[i];
        for (uint32_t r = 0; r < nrun; ++r) {
            const BatchParams &bp = d.runs[r];
            const uint32_t n = bp.n_mid;
            if (i >= n) continue;
            uint32_t x[8];
            first_bits8(bp.base, bp.nblk, p, x);
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k) bp.xfirst[size_t(k) * n + i] = x[k];
        }
    }
}

// the same for one run passed by value
__global__ void __launch_bounds__(256) k_xfirst1(BatchParams bp)
{
    const uint32_t n = bp.n_mid;
    for (uint32_t i = bp.i0 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t x[8];
        first_bits8(bp.base, bp.nblk, bp.primes[i], x);
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) bp.xfirst[size_t(k) * n + i] = x[k];
    }
}

// Tile-local first mark of a prime from its run-level first bit x.
__device__ __forceinline__ uint32_t local_start(uint32_t x, uint32_t t0, uint32_t p, uint32_t magic, uint32_t tb)
{
    if (x == kNone) return kNone;
    if (x >= t0) {
        const uint32_t d = x - t0;
        return d < tb ? d : kNone;
    }
    const uint32_t d = t0 - x;
    const uint32_t q = __umulhi(d, magic);  // floor(d / p) or one less
    uint32_t rem = d - q * p;
    if (rem >= p) rem -= p;
    return rem ? p - rem : 0;
}

// Tile-bin staging of the persistent tile kernel: the first `cap` offsets
// of an item's tile bin (cap: what the shared memory beside the tile holds,
// up to kTbStage, a multiple of kTbPiece, possibly 0) go into shared memory
// by bulk copies issued at the item's start (they land while the CTA
// sieves), the rest is prefetched into L2 by the TMA unit and read from
// there.
constexpr uint32_t kTbStage = 20480;       // offsets (80 KB), a multiple of kTbPiece
constexpr uint32_t kTbPiece = 4096;        // offsets per bulk copy (16 KB)

// thread 0 at an item's start: stages the first min(n, cap) offsets of the
// tile bin e (n offsets; the copy rounded up to 16 bytes, which stays in the
// bin: capacities are multiples of 32 offsets) into stg, completing on bar,
// and prefetches the rest into L2. Returns the offsets staged.
__device__ __forceinline__ uint32_t stage_tile_bin(uint32_t *stg, uint64_t *bar, const uint32_t *e, uint32_t n,
                                                   uint32_t cap)
{
    const uint32_t staged = min(n, cap);
    if (n > cap) bulk_prefetch_l2(e + cap, ((n - cap + 3u) & ~3u) * 4u);
    if (!staged) return 0;
    const uint32_t words = (staged + 3u) & ~3u;
    fence_proxy_async();  // the CTA's earlier reads of stg before the copies
    mbar_arrive_expect_tx(bar, words * 4u);
    for (uint32_t w0 = 0; w0 < words; w0 += kTbPiece)
        bulk_copy_g2s(stg + w0, e + w0, min(kTbPiece, words - w0) * 4u, bar);
    return staged;
}

// Clears bit b of the shared-memory tile s: ~(1 << (b mod 32)) as one
// funnel-shift rotation of ~1.
__device__ __forceinline__ void clear_bit(uint32_t *s, uint32_t b)
{
    atomicAnd(&s[b >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, b));
}

// Clears bits b, b + st, b + 2 st, ... below tl (b < tl + st, tl + 4 st < 2^32):
// four marks per bound check.
__device__ __forceinline__ void clear_stride(uint32_t *s, uint32_t b, uint32_t st, uint32_t tl)
{
    for (; b + 3u * st < tl; b += 4u * st) {
        clear_bit(s, b);
        clear_bit(s, b + st);
        clear_bit(s, b + 2u * st);
        clear_bit(s, b + 3u * st);
    }
    for (; b < tl; b += st) clear_bit(s, b);
}

// Sieves bits [t0, t0 + tl) of class array k of a run in shared memory s
// (the group patterns already in pat) and stores them: tile ti of the class
// array, tb bits per tile (the buffer s holds tb bits), tl <= tb a multiple
// of 128 bits. Ends with the CTA synchronized, s free for the next tile.
// kVec4: the context's own prime and reciprocal arrays (16-byte aligned,
// padded by 4 words), read four at a time, and the tile bin staged by
// stage_tile_bin (*nb offsets, the first min(*nb, cap) in stg once bar
// completes the phase of parity bit 0 of phase); otherwise any arrays and
// the tile bin read from global memory.
template <bool kVec4>
__device__ __forceinline__ void tile_body(const BatchParams &bp, const GroupInfo &gi, const uint32_t *pat,
                                          uint32_t *s, uint32_t k, uint32_t ti, uint32_t t0, uint32_t tl,
                                          uint32_t tb, const uint32_t *stg = nullptr, uint64_t *bar = nullptr,
                                          uint32_t *phase = nullptr, const uint32_t *nb = nullptr, uint32_t cap = 0)
{
    const uint32_t tid = threadIdx.x, bs = blockDim.x;
    const uint32_t tw = tl >> 5;
    const uint64_t q0 = bp.base + 30ull * t0 + unit30(k);

    // phase of this thread's first word in each group's canonical pattern:
    // local bit x is cleared by the group iff (x + c) mod P has a factor in
    // the group, c = (P - Y) mod P, Y = -q0 / 30 (mod P)
    uint32_t ph[kNumGroups], stp[kNumGroups];
#pragma unroll
    for (int g = 0; g < kNumGroups; ++g) {
        const uint32_t P = gi.P[g];
        const uint32_t qm = uint32_t(q0 % P);
        const uint32_t y = uint32_t(uint64_t((P - qm) % P) * gi.inv30[g] % P);
        const uint32_t c = (P - y) % P;
        ph[g] = uint32_t((32ull * tid + c) % P);
        stp[g] = uint32_t((32ull * bs) % P);
    }
    for (uint32_t w = tid; w < tw; w += bs) {
        uint32_t v = ~0u;
#pragma unroll
        for (int g = 0; g < kNumGroups; ++g) {
            const uint32_t *pg = pat + gi.off[g];
            const uint32_t x = ph[g];
            v &= __funnelshift_r(pg[x >> 5], pg[(x >> 5) + 1], x & 31);
            uint32_t nx = x + stp[g];
            if (nx >= gi.P[g]) nx -= gi.P[g];
            ph[g] = nx;
        }
        s[w] = v;
    }
    __syncthreads();
    if (tid == 0 && q0 < 4096) {
        // the pattern primes are prime themselves; 1 is not
        const uint32_t small[16] = {7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67};
        for (int i = 0; i < 16; ++i) {
            const uint32_t p = small[i];
            if (p % 30 == unit30(k) && p >= q0) {
                const uint32_t b = uint32_t((p - q0) / 30);
                if (b < tl) s[b >> 5] |= 1u << (b & 31);
            }
        }
        if (q0 == 1) s[0] &= ~1u;
    }
    __syncthreads();

    const uint32_t lane = tid & 31, warp = tid >> 5, nw = bs >> 5;
    const uint32_t *xk = bp.xfirst + size_t(k) * bp.n_mid;
    // small primes: a warp per prime, lanes take every 32nd multiple
    for (uint32_t i = bp.i0 + warp; i < bp.i_warp; i += nw) {
        const uint32_t p = bp.primes[i];
        const uint32_t l = local_start(xk[i], t0, p, bp.magic[i], tl);
        if (l >= tl) continue;
        clear_stride(s, l + lane * p, 32u * p, tl);
    }
    if constexpr (kVec4) {
        // the rest: four consecutive primes per thread and round, their
        // primes and reciprocals as one 16-byte load each and their first
        // bits as four loads, all issued before any of their marks (one L2
        // round trip per four primes)
        const uint32_t n = bp.n_mid, i_lo = bp.i_warp, c_lo = i_lo & ~3u;
        for (uint32_t i = c_lo + 4 * tid; i < n; i += 4 * bs) {
            const uint4 p4 = __ldg(reinterpret_cast<const uint4 *>(bp.primes + i));
            const uint4 m4 = __ldg(reinterpret_cast<const uint4 *>(bp.magic + i));
            uint32_t x4[4];
#pragma unroll
            for (uint32_t u = 0; u < 4; ++u) x4[u] = i + u < n ? __ldg(xk + i + u) : kNone;
            const uint32_t pv[4] = {p4.x, p4.y, p4.z, p4.w}, mv[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
            for (uint32_t u = 0; u < 4; ++u) {
                if (i + u < i_lo) continue;
                const uint32_t p = pv[u];
                const uint32_t l = local_start(x4[u], t0, p, mv[u], tl);
                if (l < tl) clear_stride(s, l, p, tl);
            }
        }
    } else {
        // the rest: a thread per prime, the next prime's three loads issued
        // before the current prime's marks
        const uint32_t *pr = bp.primes, *mg = bp.magic;
        const uint32_t n = bp.n_mid;
        uint32_t i = bp.i_warp + tid;
        uint32_t p = 0, x = kNone, m = 0;
        if (i < n) {
            p = __ldg(pr + i);
            x = __ldg(xk + i);
            m = __ldg(mg + i);
        }
        while (i < n) {
            const uint32_t j = i + bs;
            uint32_t pn = 0, xn = kNone, mn = 0;
            if (j < n) {
                pn = __ldg(pr + j);
                xn = __ldg(xk + j);
                mn = __ldg(mg + j);
            }
            const uint32_t l = local_start(x, t0, p, m, tl);
            if (l < tl) clear_stride(s, l, p, tl);
            i = j;
            p = pn;
            x = xn;
            m = mn;
        }
    }
    // a binned batch: the hit-list marks of this tile (offsets within it,
    // clamped to the tile buffer: a stale staged word or a damaged bin can
    // clear a wrong bit, never touch memory outside s)
    const uint32_t omax = tb - 1;
    if constexpr (kVec4) {
        const uint32_t n = *nb, staged = min(n, cap);
        if (staged) {
            bool ok = mbar_wait(bar, *phase & 1u, bp.spin0);
            if (!ok) {
                atomicOr(bp.err, kErrStaging);
                ok = mbar_wait(bar, *phase & 1u);
            }
            *phase ^= 1u;
            const uint4 *v4 = reinterpret_cast<const uint4 *>(stg);
            for (uint32_t i = tid; ok && 4 * i < staged; i += bs) {
                const uint4 v = v4[i];
                const uint32_t at = 4 * i;
                atomicAnd(&s[min(v.x, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v.x));
                if (at + 1 < staged) atomicAnd(&s[min(v.y, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v.y));
                if (at + 2 < staged) atomicAnd(&s[min(v.z, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v.z));
                if (at + 3 < staged) atomicAnd(&s[min(v.w, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v.w));
            }
        }
        if (n > cap) {
            // the rest from L2, four groups of four per thread in flight
            const uint32_t tile = k * bp.tb_tiles + bp.tb_vt0 + ti, m = n - cap;
            const uint4 *e = reinterpret_cast<const uint4 *>(bp.tb_buf + size_t(tile) * bp.tb_cap + cap);
            for (uint32_t i = tid; 4 * i < m; i += 4 * bs) {
                uint4 v[4];
#pragma unroll
                for (uint32_t u = 0; u < 4; ++u) {
                    const uint32_t g = i + u * bs;
                    v[u] = 4 * g < m ? __ldcs(e + g) : make_uint4(0u, 0u, 0u, 0u);
                }
#pragma unroll
                for (uint32_t u = 0; u < 4; ++u) {
                    const uint32_t at = 4 * (i + u * bs);
                    if (at < m) atomicAnd(&s[min(v[u].x, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v[u].x));
                    if (at + 1 < m) atomicAnd(&s[min(v[u].y, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v[u].y));
                    if (at + 2 < m) atomicAnd(&s[min(v[u].z, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v[u].z));
                    if (at + 3 < m) atomicAnd(&s[min(v[u].w, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v[u].w));
                }
            }
        }
    } else if (bp.tb_cap && bp.hl_quota) {
        const uint32_t tile = k * bp.tb_tiles + bp.tb_vt0 + ti;
        const uint32_t n = min(__ldcg(bp.tb_cnt + tile), bp.tb_cap);
        const uint4 *e = reinterpret_cast<const uint4 *>(bp.tb_buf + size_t(tile) * bp.tb_cap);
        // four groups of four per thread in flight before their marks
        for (uint32_t i = tid; 4 * i < n; i += 4 * bs) {
            uint4 v[4];
#pragma unroll
            for (uint32_t u = 0; u < 4; ++u) {
                const uint32_t g = i + u * bs;
                v[u] = 4 * g < n ? __ldcs(e + g) : make_uint4(0u, 0u, 0u, 0u);
            }
#pragma unroll
            for (uint32_t u = 0; u < 4; ++u) {
                const uint32_t at = 4 * (i + u * bs);
                if (at < n) atomicAnd(&s[min(v[u].x, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v[u].x));
                if (at + 1 < n) atomicAnd(&s[min(v[u].y, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v[u].y));
                if (at + 2 < n) atomicAnd(&s[min(v[u].z, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v[u].z));
                if (at + 3 < n) atomicAnd(&s[min(v[u].w, omax) >> 5], __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v[u].w));
            }
        }
    }
    __syncthreads();
    uint4 *dst = reinterpret_cast<uint4 *>(bp.map + size_t(k) * bp.wpc + (t0 >> 5));
    const uint4 *src = reinterpret_cast<const uint4 *>(s);
    for (uint32_t i = tid; i < tw / 4; i += bs) dst[i] = src[i];
    __syncthreads();
}

// Persistent tile kernel: CTAs take the batch's (run, class, tile) items
// from a work counter; tiles of tb bits (a multiple of 128), a run's last
// tile of a class ends at its class array's end; up to kCap offsets of each
// tile bin staged into shared memory. kCap is a compile-time constant: with
// it as a runtime parameter the kernel measured 3.7 times slower (47.9
// against 13.05 ms per 128-segment batch at 2^20-bit tiles, one GB300).
template <uint32_t kCap>
__global__ void __launch_bounds__(1024, 1) k_tile(BatchDesc d, GroupInfo gi, uint32_t tb)
{
    constexpr uint32_t cap = kCap;
    // shared memory: the tile, the tile-bin staging buffer, the patterns
    extern __shared__ __align__(16) uint32_t sm_tile[];
    uint32_t *s = sm_tile;
    uint32_t *stg = sm_tile + (tb >> 5);
    uint32_t *pat = stg + cap;
    const uint32_t nrun = d.h->nrun, items = d.h->tile_items;
    if (!nrun) return;
    __shared__ uint32_t s_j, s_nb;
    __shared__ uint64_t s_bar;
    if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        mbar_init_fence();
    }
    uint32_t phase = 0;
    for (uint32_t i = threadIdx.x; i < gi.words; i += blockDim.x) pat[i] = d.runs[0].pat[i];
    for (;;) {
        const uint32_t j = next_item(d.work + kWorkTile, &s_j);  // synchronizes the CTA
        if (j >= items) break;
        const uint32_t r = find_prefix(d.tile_pref, nrun, j);
        const BatchParams &bp = d.runs[r];
        // items tile-major within a run: a tile's eight classes side by side,
        // so the tiles of one segment are one range of items
        const uint32_t local = j - __ldg(d.tile_pref + r);
        const uint32_t k = local & 7u, ti = local >> 3, t0 = ti * tb;
        const uint32_t tl = min(tb, bp.wpc * 32 - t0);
        if (threadIdx.x == 0) {
            uint32_t n = 0;
            if (bp.tb_cap && bp.hl_quota) {
                const uint32_t tile = k * bp.tb_tiles + bp.tb_vt0 + ti;
                n = min(__ldcg(bp.tb_cnt + tile), bp.tb_cap);
                stage_tile_bin(stg, &s_bar, bp.tb_buf + size_t(tile) * bp.tb_cap, n, cap);
            }
            s_nb = n;
        }
        tile_body<true>(bp, gi, pat, s, k, ti, t0, tl, tb, stg, &s_bar, &phase, &s_nb, cap);
    }
}

// the staging capacities the host chooses from (the largest that fits)
constexpr uint32_t kTbStages[3] = {kTbStage, 2 * kTbPiece, 0};
template __global__ void k_tile<kTbStages[0]>(BatchDesc, GroupInfo, uint32_t);
template __global__ void k_tile<kTbStages[1]>(BatchDesc, GroupInfo, uint32_t);
template __global__ void k_tile<kTbStages[2]>(BatchDesc, GroupInfo, uint32_t);

// one run by value: grid (tiles_pc, 8), full tiles (wpc = tiles_pc tiles)
__global__ void __launch_bounds__(1024, 1) k_tile1(BatchParams bp, GroupInfo gi)
{
    extern __shared__ uint32_t sm[];
    const uint32_t tb = 1u << bp.tile_log2;
    uint32_t *pat = sm + (tb >> 5);
    for (uint32_t i = threadIdx.x; i < gi.words; i += blockDim.x) pat[i] = bp.pat[i];
    __syncthreads();
    tile_body<false>(bp, gi, pat, sm, blockIdx.y, blockIdx.x, blockIdx.x << bp.tile_log2, tb, tb);
}

// The packed large-prime tier (the reference's pack_large_primes,
// decode_large and large_packed_body, src/host_math.cpp:187-209,
// kernels/goldbach.cl:1678-1829 with the wheel walk of 638-748, in this
// repository's own form): the primes of [p_mid, p_hl) stream at one byte per
// prime, a half gap (p_i - p_{i-1}) / 2, with the first prime of every group
// of kPackGroup primes in a table of its own; a warp decodes a group (lane
// l: eight primes, its gap bytes as one 8-byte load, the group's running sum
// by a warp scan). Each prime then marks every run it reaches, class by
// class: the multiples q = p m of class k are the bits t0, t0 + p, t0 + 2 p,
// ... with m = m0 + 30 j. Multipliers with a factor 7, 11 or 13 are stepped
// over by a wheel mod 7 * 11 * 13 = 1001 (720 steps in 1001; inside one class
// array this is the reference's 30030 wheel, whose factor 30 the class
// layout already holds); multipliers with a factor 17..43 are skipped by a
// test of their residues, four 8-bit lanes per word. Either way q has a prime
// factor the pattern stage clears. A mark reads the word and clears the bit
// with an atomic AND only if it is still set.
constexpr uint32_t kWheelUnits = 720;          // residues mod 1001 coprime to it
constexpr uint32_t kSkipLanes1 = 0x1D171311u;  // 17, 19, 23, 29 as bytes
constexpr uint32_t kSkipLanes2 = 0x2B29251Fu;  // 31, 37, 41, 43
constexpr uint32_t kSkipBias1 = 0x63696D6Fu;   // 128 - 17, 128 - 19, 128 - 23, 128 - 29
constexpr uint32_t kSkipBias2 = 0x55575B61u;   // 128 - 31, 128 - 37, 128 - 41, 128 - 43

// per byte lane, (x + d) mod f for lanes x < f and d <= 4: add, then subtract
// f where the sum reached f (the bias 128 - f carries that into bit 7)
__device__ __forceinline__ uint32_t lanes_step(uint32_t x, uint32_t d, uint32_t f, uint32_t bias)
{
    x += d * 0x01010101u;
    const uint32_t ge = ((x + bias) >> 7) & 0x01010101u;
    return x - ((ge * 0xFFu) & f);
}

// nonzero iff some byte lane of x is zero
__device__ __forceinline__ uint32_t lanes_zero(uint32_t x) { return (x - 0x01010101u) & ~x & 0x80808080u; }

// Marks the multiples of p in one class array wk of nblk bits from bit t on.
// c = m0 / 30 mod 1001 and the lanes r1 (17..29), r2 (31..43) = m0 / 30 mod
// f for the multiplier m0 of bit t, so that m0 + 30 j has the factor f iff
// (c + j) or lane f of r + j is 0 mod f. wheel[x], x < 1001: the rank of the
// first unit >= x (wrapping) | its distance << 10; wheel[1001 + rank]: the
// gap from that unit to the next.
__device__ __forceinline__ void large_walk(uint32_t *wk, uint32_t nblk, uint32_t t, uint32_t p, uint32_t c,
                                           uint32_t r1, uint32_t r2, const uint16_t *wheel)
{
    const uint32_t e = wheel[c];
    uint32_t rank = e & 1023u;
    const uint32_t d0 = e >> 10;
    if (d0) {
        if (uint64_t(nblk - t) <= uint64_t(d0) * p) return;
        t += d0 * p;
        r1 = lanes_step(r1, d0, kSkipLanes1, kSkipBias1);
        r2 = lanes_step(r2, d0, kSkipLanes2, kSkipBias2);
    }
    for (;;) {
        if (!(lanes_zero(r1) | lanes_zero(r2))) {
            uint32_t *a = wk + (t >> 5);
            const uint32_t bit = 1u << (t & 31);
            if (__ldcg(a) & bit) atomicAnd(a, ~bit);
        }
        const uint32_t g = wheel[kWheelM + rank];
        if (uint64_t(nblk - t) <= uint64_t(g) * p) break;
        t += g * p;
        rank = rank + 1 == kWheelUnits ? 0u : rank + 1;
        r1 = lanes_step(r1, g, kSkipLanes1, kSkipBias1);
        r2 = lanes_step(r2, g, kSkipLanes2, kSkipBias2);
    }
}

// The packed large primes [n_mid, n_hl) of every run: a CTA per item of 32
// consecutive primes, a thread per (prime, class) walk, so that every walk of
// a batch (about eight per prime) runs side by side (the walks wait on
// global memory; a thread per prime walking its classes in turn measured
// about half the pipeline's speed with 46 K primes on this tier). Warp 0
// decodes the item's packing group (lane l: eight primes from one 8-byte
// load, the group's running sum by a warp scan) into shared memory.
constexpr uint32_t kLargeItem = 32;  // primes per CTA item; kPackGroup / kLargeItem items per group
__global__ void __launch_bounds__(256) k_large(BatchDesc d)
{
    __shared__ uint16_t s_wheel[kWheelTabWords];
    __shared__ uint32_t s_p[kLargeItem];
    const uint32_t nrun = d.h->nrun;
    if (!nrun) return;
    const BatchParams &b0 = d.runs[0];
    // runs whose large range is empty may have n_mid below the stream's start
    const uint32_t lo = max(d.h->n_mid_min, b0.pk_i0), hi = d.h->n_hl_max;
    if (lo >= hi) return;
    for (uint32_t i = threadIdx.x; i < kWheelTabWords; i += blockDim.x) s_wheel[i] = b0.wheel[i];
    const uint16_t *s_inv = s_wheel + kWheelM + kWheelUnits;  // x^-1 mod 1001 (0: none)
    const uint16_t *s_invf = s_inv + kWheelM;                  // x^-1 mod f, f = 17..43 back to back
    constexpr uint32_t kF[8] = {17, 19, 23, 29, 31, 37, 41, 43};
    constexpr uint32_t kFo[8] = {0, 17, 36, 59, 88, 119, 156, 197};
    const uint32_t tid = threadIdx.x, lane = tid & 31, i0 = b0.pk_i0;
    const uint32_t j_lo = (lo - i0) / kLargeItem, j_hi = (hi - i0 + kLargeItem - 1) / kLargeItem;
    const uint32_t k = tid & 7;        // this thread's class
    const uint32_t slot = tid >> 3;    // and prime of the item
    for (uint32_t j = j_lo + blockIdx.x; j < j_hi; j += gridDim.x) {
        __syncthreads();  // the wheel table loaded; the last item's primes read
        if (tid < 32) {
            const uint32_t g = j / (kPackGroup / kLargeItem), sl = j % (kPackGroup / kLargeItem);
            const uint2 gv = __ldg(reinterpret_cast<const uint2 *>(b0.pk_gap) + size_t(g) * (kPackGroup / 8) + lane);
            uint32_t sum = 0;
#pragma unroll
            for (uint32_t b = 0; b < 32; b += 8) sum += ((gv.x >> b) & 0xFFu) + ((gv.y >> b) & 0xFFu);
            uint32_t incl = sum;
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(~0u, incl, o);
                if (lane >= o) incl += y;
            }
            uint32_t p = __ldg(b0.pk_base + g) + 2u * (incl - sum);
            const uint32_t first = sl * (kLargeItem / 8);  // the lanes of this item's slice of the group
#pragma unroll
            for (uint32_t u = 0; u < 8; ++u) {
                p += 2u * (((u < 4 ? gv.x : gv.y) >> (8 * (u & 3))) & 0xFFu);
                if (lane >= first && lane < first + kLargeItem / 8) s_p[(lane - first) * 8 + u] = p;
            }
        }
        __syncthreads();
        const uint32_t i = i0 + j * kLargeItem + slot;
        if (i < lo || i >= hi) continue;
        const uint32_t p = s_p[slot];
        const float rp = __frcp_rn(float(p));
        const uint32_t iv = inv30_mod(p);
        const uint32_t uk = unit30(k);
        const uint32_t ck = mod_below(uint64_t(uk) * iv, p, rp);  // u_k / 30 mod p
        // (30 p)^-1 mod 1001 and mod each skip prime f
        const uint32_t a1001 = s_inv[30u * (p % kWheelM) % kWheelM];
        uint32_t af[8];
#pragma unroll
        for (uint32_t jj = 0; jj < 8; ++jj) af[jj] = s_invf[kFo[jj] + 30u * (p % kF[jj]) % kF[jj]];
        for (uint32_t ri = 0; ri < nrun; ++ri) {
            const BatchParams &bp = d.runs[ri];
            if (i < bp.n_mid || i >= bp.n_hl) continue;
            // run 0's window (the plain form's per-segment launches):
            // bits [b0, b1), b0 a multiple of 32, as a run of its own
            const uint32_t w0 = ri ? 0u : d.h->win_b0, w1 = ri ? bp.nblk : min(bp.nblk, d.h->win_b1);
            if (w0 >= w1) continue;
            const uint64_t base = bp.base + 30ull * w0;
            const uint32_t nblk = w1 - w0;
            const uint32_t r = mod_u64(base, p, rp);
            // t_k = -(base + u_k) / 30 mod p = tb - c_k, tb = -base / 30
            const uint32_t tb = mod_below(uint64_t(r ? p - r : 0) * iv, p, rp);
            uint32_t tk = tb >= ck ? tb - ck : tb + (p - ck);
            if (uint64_t(p) * p > base) {  // only near the bottom of the range: q >= p^2
                const uint64_t pp = uint64_t(p) * p;
                const uint64_t q = base + 30ull * tk + uk;
                if (q < pp) {
                    const uint64_t tmin = (pp - base - uk + 29) / 30;
                    const uint64_t tt = tk + (tmin - tk + p - 1) / p * p;
                    tk = tt < nblk ? uint32_t(tt) : kNone;
                }
            }
            if (tk >= nblk) continue;
            // m0 = q0 / p with q0 = base + 30 tk + u_k, so m0 / 30 = q0 (30 p)^-1
            // mod 1001 and mod f (the run base's residues, moved to the window)
            const uint32_t bm1 = (bp.bm1 + 30u * (w0 % kWheelM)) % kWheelM;
            const uint32_t c = (bm1 + 30u * (tk % kWheelM) + uk) % kWheelM * a1001 % kWheelM;
            uint32_t r1 = 0, r2 = 0;
#pragma unroll
            for (uint32_t jj = 0; jj < 8; ++jj) {
                const uint32_t f = kF[jj];
                const uint32_t bf = (uint32_t(bp.bres[jj]) + 30u * (w0 % f)) % f;
                const uint32_t q = (bf + 30u * (tk % f) + uk) % f;
                const uint32_t rho = q * af[jj] % f;
                if (jj < 4) r1 |= rho << (8 * jj);
                else r2 |= rho << (8 * (jj - 4));
            }
            large_walk(bp.map + size_t(k) * bp.wpc + (w0 >> 5), nblk, tk, p, c, r1, r2, s_wheel);
        }
    }
}

// floor(x / p) and x mod p for any 64-bit x and 2^7 <= p < 2^32, without a
// division: two base-2^32 digits, each remainder by mod_below, each digit
// of the quotient exactly as (digit - remainder) * p^-1 mod 2^32 (the
// quotient digit is below 2^32, so the multiple of p divides exactly).
__device__ __forceinline__ uint64_t divmod_u64(uint64_t x, uint32_t p, float rp, uint32_t pinv, uint32_t &rem)
{
    const uint32_t hi = uint32_t(x >> 32), lo = uint32_t(x);
    const uint32_t rh = hi < p ? hi : mod_below(hi, p, rp);
    const uint32_t qh = (hi - rh) * pinv;
    const uint64_t x2 = (uint64_t(rh) << 32) | lo;
    rem = mod_below(x2, p, rp);
    const uint32_t ql = uint32_t(x2 - rem) * pinv;
    return (uint64_t(qh) << 32) | ql;
}

// p^-1 mod 2^32 for odd p (Newton: the correct low bits double each step)
__device__ __forceinline__ uint32_t inv_mod_2_32(uint32_t p)
{
    uint32_t x = p;  // p * p = 1 (mod 8)
#pragma unroll
    for (int i = 0; i < 4; ++i) x *= 2u - p * x;
    return x;
}

// Hit lists through the prime-multiplier table (the reference's mt_build /
// hl_harvest_mt / hl_apply, kernels/goldbach.cl:3181-3471): for a prime
// p >= cbrt(q), a composite multiplier m of q = p m has a prime factor below
// p, which marks q already, so only prime m matter. One thread per prime
// p and run: the primes m in [ceil(Q0 / p), floor(Q1 / p)] are one
// contiguous run of bytes of the table; each gives q = p m, whose class bit
// is cleared with an atomic AND. Every such q is a semiprime whose factors
// are both above the sieving bound of the other stages, so the bit is set
// and no read is needed.
__device__ __forceinline__ void ovf_push(const BatchParams &bp, uint32_t k, uint32_t t)
{
    const uint32_t slot = atomicAdd(bp.ovf_cnt, 1u);
    if (slot < bp.ovf_cap) bp.ovf_buf[slot] = make_uint2(k, t);
}

// direct = 0: a binned batch's harvest (launched before the tiles); direct =
// 1: every other batch's direct marks (launched after the tiles)
__global__ void __launch_bounds__(256) k_hitlist(BatchDesc d, uint32_t direct)
{
    const uint32_t nrun = d.h->nrun;
    if (!nrun) return;
    const bool binned = hl_binned(d.runs[0]);
    if (binned == (direct != 0)) return;
    // per (class of p, class of m): the class kq of q = p m, its residue
    // u_kq and u_m, as kq | u_kq << 8 | u_m << 16; the class of a residue
    __shared__ uint32_t s_cls[8][8];
    __shared__ uint8_t s_res[32];
    if (threadIdx.x < 64) {
        const uint32_t a = threadIdx.x >> 3, b = threadIdx.x & 7;
        const uint32_t uq = unit30(a) * unit30(b) % 30;
        s_cls[a][b] = class_of(uq) | (uq << 8) | (unit30(b) << 16);
    } else if (threadIdx.x < 96) {
        s_res[threadIdx.x - 64] = uint8_t(class_of(threadIdx.x - 64));
    }
    __shared__ uint32_t s_hcnt[kHlMaxBins];
    if (threadIdx.x < kHlMaxBins) s_hcnt[threadIdx.x] = 0;
    __syncthreads();
    // a binned batch files its marks in region bins (k_binsort takes them on)
    const BatchParams &run0 = d.runs[0];
    const uint32_t quota = binned ? run0.hl_quota : 0u;
    const uint32_t rlog = run0.hl_rlog, nreg = run0.hl_nreg, nbin = 8 * nreg;
    uint32_t *const hl_mine = quota ? run0.hl_buf + size_t(blockIdx.x) * nbin * quota : nullptr;
    // bit r set for the units r mod 30: the classes below a residue
    constexpr uint32_t kUnits = (1u << 1) | (1u << 7) | (1u << 11) | (1u << 13) | (1u << 17) | (1u << 19) |
                                (1u << 23) | (1u << 29);
    constexpr uint32_t kInv15 = 0xEEEEEEEFu;  // 15^-1 mod 2^32
    const uint32_t *primes = d.runs[0].primes;
    const uint32_t nhi = d.h->n_all_max;
    for (uint32_t i = d.h->n_hl_min + blockIdx.x * blockDim.x + threadIdx.x; i < nhi;
         i += gridDim.x * blockDim.x) {
        const uint32_t p = primes[i];
        const float rp = __frcp_rn(float(p));
        const uint32_t pinv = inv_mod_2_32(p);
        const uint32_t kp = s_res[p % 30];
        for (uint32_t ri = 0; ri < nrun; ++ri) {
            const BatchParams &bp = d.runs[ri];
            if (i < bp.n_hl || i >= bp.n_all) continue;
            const uint64_t base = bp.base;
            // m in [ceil(base / p), floor(q1 / p)], q1 = base + span: the
            // second quotient from the first and a division of r0 + span < 2^37
            uint32_t r0;
            const uint64_t qb = divmod_u64(base, p, rp, pinv, r0);
            const uint64_t span = 30ull * bp.nblk - 1;
            // a run narrower than p (most pairs of a batch of short windows)
            // holds a multiple of p only if r0 is 0 or above p - span
            if (span < p && r0 && p - r0 > span) continue;
            const uint64_t x = uint64_t(r0) + span;
            const uint32_t r1 = mod_below(x, p, rp);
            const uint64_t mlo = qb + (r0 ? 1 : 0), mhi = qb + uint32_t(x - r1) * pinv;
            if (mhi < mlo) continue;
            const uint64_t m0 = bp.m0;
            if (mlo < m0 || mhi > bp.m1) {
                atomicOr(bp.err, kErrTable);
                continue;
            }
            uint32_t *map = bp.map;
            const uint32_t wpc = bp.wpc;
            const uint32_t *mtab = bp.mtab;
            const uint32_t vbase = bp.tb_vt0 * run0.tile_bits;  // the run's first virtual bit (binned)
            // table bytes b0..b1; in the end bytes only the classes inside [mlo, mhi]
            const uint64_t b0 = (mlo - m0) / 30, b1 = (mhi - m0) / 30;
            const uint32_t dl = uint32_t(mlo - m0 - 30 * b0), dh = uint32_t(mhi - m0 - 30 * b1);
            const uint32_t lo_byte = (0xFFu << __popc(kUnits & ((1u << dl) - 1u))) & 0xFFu;
            const uint32_t hi_byte = (1u << __popc(kUnits & ((2u << dh) - 1u))) - 1u;
            const uint64_t w0 = b0 >> 2, w1 = b1 >> 2;
            const uint32_t lo_mask = (0xFFFFFFFFu << (8 * (b0 & 3))) & ~(0xFFu << (8 * (b0 & 3))) |
                                     (lo_byte << (8 * (b0 & 3)));
            const uint32_t hi_shift = 8 * uint32_t(b1 & 3);
            const uint32_t hi_mask = (hi_shift ? (0xFFFFFFFFu >> (32 - hi_shift)) : 0u) | (hi_byte << hi_shift);
            // q - base - u_q = xw + p (30 jb + u_m) - u_q for byte jb of word
            // w, xw = p (m0 + 120 w) - base: a multiple of 30 below 2^64, and
            // the class bit t = that / 30 < 2^31, so its low 32 bits suffice:
            // bits 1..32 of it times 15^-1 mod 2^32
            const uint32_t *tw = mtab + w0;
            const uint32_t nw = uint32_t(w1 - w0);
            const uint64_t step = 120ull * p;
            uint64_t xw = uint64_t(p) * m0 - base + step * w0;
            // the next table word loaded before this word's marks (its
            // latency hidden behind them)
            uint32_t vnext = __ldg(tw);
            for (uint32_t iw = 0; iw <= nw; ++iw, xw += step) {
                uint32_t v = vnext;
                if (iw < nw) vnext = __ldg(tw + iw + 1);
                if (iw == 0) v &= lo_mask;
                if (iw == nw) v &= hi_mask;
                while (v) {
                    const uint32_t j = __ffs(v) - 1u;
                    v &= v - 1u;
                    const uint32_t e = s_cls[kp][j & 7];
                    const uint64_t xq = xw + uint64_t(p) * (30u * (j >> 3) + (e >> 16)) - ((e >> 8) & 0xFFu);
                    const uint32_t t = uint32_t(xq >> 1) * kInv15;
                    if (quota) {
                        const uint32_t v = vbase + t;
                        const uint32_t bin = (e & 0xFFu) * nreg + (v >> rlog);
                        const uint32_t pos = atomicAdd(&s_hcnt[bin], 1u);
                        if (pos < quota) hl_mine[size_t(bin) * quota + pos] = v & ((1u << rlog) - 1u);
                        else ovf_push(run0, e & 0xFFu, v);
                        continue;
                    }
                    atomicAnd(map + size_t(e & 0xFFu) * wpc + (t >> 5), ~(1u << (t & 31)));
                }
            }
        }
    }
    if (quota) {
        __syncthreads();
        for (uint32_t b = threadIdx.x; b < nbin; b += blockDim.x) run0.hl_cnt[blockIdx.x * nbin + b] = s_hcnt[b];
    }
}

// exclusive prefix sums of in[0, n) into out (n <= 4 * 256; 256 threads;
// the caller synchronises before reading out or reusing s_wsum)
__device__ __forceinline__ void block_excl_scan4(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *s_wsum)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t v[4], sum = 0;
#pragma unroll
    for (uint32_t j = 0; j < 4; ++j) {
        const uint32_t idx = 4 * tid + j;
        v[j] = idx < n ? in[idx] : 0u;
        sum += v[j];
    }
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(~0u, x, o);
        if (lane >= uint32_t(o)) x += y;
    }
    if (lane == 31) s_wsum[warp] = x;
    __syncthreads();
    uint32_t run = x - sum;
    for (uint32_t i = 0; i < warp; ++i) run += s_wsum[i];
#pragma unroll
    for (uint32_t j = 0; j < 4; ++j) {
        const uint32_t idx = 4 * tid + j;
        if (idx < n) out[idx] = run;
        run += v[j];
    }
}

constexpr uint32_t kSortPer = 16;                   // offsets per thread and chunk (four uint4)
constexpr uint32_t kSortChunk = 256 * kSortPer;     // offsets a CTA sorts in shared memory at a time

// Binned hit lists, sorted by tile: every (harvest CTA, region bin) list,
// kSortChunk offsets at a time (read once, into registers), is counted per
// tile of its region, given room in each tile's bin by one atomic add per
// tile, sorted by tile in shared memory and stored tile run by tile run
// (consecutive threads, consecutive addresses). Offsets beyond a tile bin's
// capacity go to the overflow list. The lists start 16-byte aligned (the
// quota is a multiple of 32 words).
// Six CTAs per SM (40 registers): the hit-list stage took 8.0 ms per
// 128-segment batch against 8.2 at four (one wave of persistent CTAs).
__global__ void __launch_bounds__(256, 6) k_binsort(BatchDesc d)
{
    __shared__ uint32_t s_out[kSortChunk];
    __shared__ uint32_t s_cnt[kSortMaxTiles], s_start[kSortMaxTiles], s_gbase[kSortMaxTiles];
    __shared__ uint32_t s_wsum[8];
    __shared__ uint32_t s_j;
    if (!hl_binned(d.runs[0])) return;
    const BatchParams &bp = d.runs[0];
    const uint32_t tid = threadIdx.x, bs = blockDim.x;
    const uint32_t quota = bp.hl_quota, nreg = bp.hl_nreg, nbin = 8 * nreg, ctas = bp.hl_ctas;
    const uint32_t rlog = bp.hl_rlog, tb = bp.tile_bits, rcp = bp.tile_rcp;
    const uint32_t items = nbin * ctas, cap = bp.tb_cap;
    for (;;) {
        const uint32_t j = next_item(d.work + kWorkBinsort, &s_j);
        if (j >= items) break;
        const uint32_t bin = j / ctas, c = j - bin * ctas;
        const uint32_t k = bin / nreg, reg = bin - k * nreg;
        const uint32_t n = min(bp.hl_cnt[size_t(c) * nbin + bin], quota);
        const uint32_t *e = bp.hl_buf + (size_t(c) * nbin + bin) * quota;
        // the region's bits [rb, rb + 2^rlog) meet tiles ti0 .. ti0 + tpr - 1
        // of the class array (tiles may straddle regions: their bins are
        // filled by every region that meets them)
        const uint32_t rb = reg << rlog;
        const uint32_t ti0 = tile_of(rb, tb, rcp);
        const uint32_t tpr = tile_of(min(rb + ((1u << rlog) - 1u), bp.tb_tiles * tb - 1), tb, rcp) - ti0 + 1;
        const uint32_t tile0 = k * bp.tb_tiles + ti0;
        for (uint32_t cs = 0; cs < n; cs += kSortChunk) {
            const uint32_t m = min(n - cs, kSortChunk);
            for (uint32_t t = tid; t < tpr; t += bs) s_cnt[t] = 0;
            // this thread's offsets: groups of four at tid + 256 u (kNone past the end)
            uint32_t v[kSortPer];
            const uint4 *e4 = reinterpret_cast<const uint4 *>(e + cs);
#pragma unroll
            for (uint32_t u = 0; u < kSortPer / 4; ++u) {
                const uint32_t g = tid + bs * u;
                const uint4 q = 4 * g < m ? __ldcs(e4 + g) : make_uint4(kNone, kNone, kNone, kNone);
                v[4 * u] = q.x;
                v[4 * u + 1] = 4 * g + 1 < m ? q.y : kNone;
                v[4 * u + 2] = 4 * g + 2 < m ? q.z : kNone;
                v[4 * u + 3] = 4 * g + 3 < m ? q.w : kNone;
            }
            __syncthreads();
            // each offset as (tile of the region, bit in the tile): t - ti0 in
            // the top 11 bits, the bit (< tb <= 2^21) in the low 21
#pragma unroll
            for (uint32_t u = 0; u < kSortPer; ++u)
                if (v[u] != kNone) {
                    const uint32_t t = rb + v[u], ti = tile_of(t, tb, rcp);
                    v[u] = ((ti - ti0) << 21) | (t - ti * tb);
                    atomicAdd(&s_cnt[v[u] >> 21], 1u);
                }
            __syncthreads();
            block_excl_scan4(s_cnt, s_start, tpr, s_wsum);
            __syncthreads();
            for (uint32_t t = tid; t < tpr; t += bs) {
                const uint32_t cn = s_cnt[t];
                s_gbase[t] = cn ? atomicAdd(bp.tb_cnt + tile0 + t, cn) : 0u;
                s_cnt[t] = s_start[t];
            }
            __syncthreads();
#pragma unroll
            for (uint32_t u = 0; u < kSortPer; ++u)
                if (v[u] != kNone) s_out[atomicAdd(&s_cnt[v[u] >> 21], 1u)] = v[u];
            __syncthreads();
            for (uint32_t i = tid; i < m; i += bs) {
                const uint32_t off = s_out[i], t = off >> 21, bit = off & ((1u << 21) - 1u);
                const uint32_t pos = s_gbase[t] + (i - s_start[t]);
                if (pos < cap) bp.tb_buf[size_t(tile0 + t) * cap + pos] = bit;
                else ovf_push(bp, k, (ti0 + t) * tb + bit);
            }
            __syncthreads();
        }
    }
}

// The overflow list of a binned batch, cleared after the tiles.
__global__ void __launch_bounds__(256) k_hl_overflow(BatchDesc d)
{
    const uint32_t nrun = d.h->nrun;
    if (!nrun || !hl_binned(d.runs[0])) return;
    const BatchParams &bp0 = d.runs[0];
    const uint32_t cnt = *bp0.ovf_cnt, tb = bp0.tile_bits;
    if (cnt > bp0.ovf_cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(bp0.err, kErrHlOverflow);
    const uint32_t n = min(cnt, bp0.ovf_cap);
    const uint32_t b0 = d.h->win_b0, b1 = d.h->win_b1;  // the plain form's window of run 0 (else everything)
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint2 e = bp0.ovf_buf[i];
        // the run of virtual bit e.y: the last one whose first virtual tile is at or below it
        const uint32_t vt = e.y / tb;
        uint32_t lo = 0, hi = nrun - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (d.runs[mid].tb_vt0 <= vt) lo = mid;
            else hi = mid - 1;
        }
        const BatchParams &bp = d.runs[lo];
        const uint32_t t = e.y - bp.tb_vt0 * tb;
        if (t < bp.nblk && t >= b0 && t < b1)
            atomicAnd(bp.map + size_t(e.x) * bp.wpc + (t >> 5), ~(1u << (t & 31)));
    }
}

// The class arrays of a sieved range, rewritten as one byte per block of 30
// (bit k = class k): one thread per class-array word, 32 bytes out.
__global__ void __launch_bounds__(256) k_wheel_bytes(BatchParams bp, uint32_t *out)
{
    const uint32_t nw = (bp.nblk + 31) / 32;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
        uint32_t a[8];
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) a[k] = bp.map[size_t(k) * bp.wpc + w];
        const uint32_t valid = (w + 1) * 32 <= bp.nblk ? 32u : bp.nblk - w * 32;
#pragma unroll
        for (uint32_t o = 0; o < 8; ++o) {
            uint32_t word = 0;
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j) {
                const uint32_t b = 4 * o + j;
                uint32_t byte = 0;
#pragma unroll
                for (uint32_t k = 0; k < 8; ++k) byte |= ((a[k] >> b) & 1u) << k;
                if (b >= valid) byte = 0;
                word |= byte << (8 * j);
            }
            out[size_t(w) * 8 + o] = word;
        }
    }
}

// Map self-check: every word of every run's class arrays in two batch
// descriptors of the same geometry (the maps built with and without hit
// lists); differing words are counted and flag the batch.
__global__ void __launch_bounds__(256) k_map_compare(BatchDesc a, BatchDesc b, uint32_t *count)
{
    const uint32_t nrun = a.h->nrun;
    for (uint32_t r = 0; r < nrun; ++r) {
        const BatchParams &ra = a.runs[r];
        const uint32_t *mb = b.runs[r].map;
        const size_t words = size_t(8) * ra.wpc;
        uint32_t bad = 0;
        for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < words; i += size_t(gridDim.x) * blockDim.x)
            bad += ra.map[i] != mb[i];
        bad = __reduce_add_sync(~0u, bad);
        if ((threadIdx.x & 31) == 0 && bad) {
            atomicAdd(count, bad);
            atomicOr(ra.err, kErrSelfCheck);
        }
    }
}

}  // namespace gbk

namespace gbh {

void launch_map_compare(const gbk::BatchDesc &a, const gbk::BatchDesc &b, uint32_t *count, const Grids &g,
                        cudaStream_t st)
{
    gbk::k_map_compare<<<g.sm * 8, 256, 0, st>>>(a, b, count);
}

static size_t tile_smem(uint32_t tile_bits, const gbk::GroupInfo &gi)
{
    return size_t((tile_bits >> 5) + gi.words) * 4;
}

// the persistent tile kernel adds the tile-bin staging buffer (stage offsets)
static size_t tile_smem_staged(uint32_t tile_bits, uint32_t stage, const gbk::GroupInfo &gi)
{
    return tile_smem(tile_bits, gi) + size_t(stage) * 4;
}

bool tile_attributes(uint32_t tile_bits, uint32_t tile_log2, const gbk::GroupInfo &gi, int device, uint32_t *stage)
{
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, gbk::k_tile<gbk::kTbStages[0]>);
    const size_t room = size_t(optin) > fa.sharedSizeBytes ? size_t(optin) - fa.sharedSizeBytes : 0;
    const size_t base = tile_smem(tile_bits, gi);
    if (base > room) return false;
    // the largest staging buffer of the kernel's instantiations that fits
    uint32_t c = 0;
    while (c < 2 && base + size_t(gbk::kTbStages[c]) * 4 > room) ++c;
    *stage = gbk::kTbStages[c];
    const int bytes = int(tile_smem_staged(tile_bits, *stage, gi));
    if (c == 0) cudaFuncSetAttribute(gbk::k_tile<gbk::kTbStages[0]>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (c == 1) cudaFuncSetAttribute(gbk::k_tile<gbk::kTbStages[1]>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (c == 2) cudaFuncSetAttribute(gbk::k_tile<gbk::kTbStages[2]>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(gbk::k_tile1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(tile_smem(1u << tile_log2, gi)));
    return true;
}

void launch_xfirst(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st)
{
    gbk::k_xfirst<<<g.sm * 8, 256, 0, st>>>(d);
}

void launch_tile(const gbk::BatchDesc &d, const gbk::GroupInfo &gi, uint32_t tile_bits, uint32_t stage,
                 const Grids &g, cudaStream_t st)
{
    const size_t bytes = tile_smem_staged(tile_bits, stage, gi);
    if (stage == gbk::kTbStages[0]) gbk::k_tile<gbk::kTbStages[0]><<<g.sm, 1024, bytes, st>>>(d, gi, tile_bits);
    else if (stage == gbk::kTbStages[1]) gbk::k_tile<gbk::kTbStages[1]><<<g.sm, 1024, bytes, st>>>(d, gi, tile_bits);
    else gbk::k_tile<gbk::kTbStages[2]><<<g.sm, 1024, bytes, st>>>(d, gi, tile_bits);
}

void launch_large(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st)
{
    gbk::k_large<<<g.sm * 8, 256, 0, st>>>(d);
}

void launch_hitlist(const gbk::BatchDesc &d, bool direct, const Grids &g, cudaStream_t st)
{
    gbk::k_hitlist<<<g.sm * g.hitlist, 256, 0, st>>>(d, direct ? 1u : 0u);
}

// the harvest's grid is one wave of resident CTAs: its primes are dealt out
// by CTA, so a second partial wave would run at a fraction of the occupancy
void query_sieve_grids(Grids &g)
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gbk::k_hitlist, 256, 0);
    g.hitlist = n > 0 ? n : 1;
}

void launch_binsort(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st)
{
    gbk::k_binsort<<<g.sm * 6, 256, 0, st>>>(d);
}

void launch_hl_overflow(const gbk::BatchDesc &d, const Grids &g, cudaStream_t st)
{
    gbk::k_hl_overflow<<<g.sm * 2, 256, 0, st>>>(d);
}

void launch_xfirst1(const gbk::BatchParams &bp, cudaStream_t st)
{
    if (bp.n_mid <= bp.i0) return;
    const uint32_t n = bp.n_mid - bp.i0;
    uint32_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    gbk::k_xfirst1<<<blocks, 256, 0, st>>>(bp);
}

void launch_tile1(const gbk::BatchParams &bp, const gbk::GroupInfo &gi, cudaStream_t st)
{
    dim3 grid(bp.tiles_pc, 8);
    gbk::k_tile1<<<grid, 1024, tile_smem(1u << bp.tile_log2, gi), st>>>(bp, gi);
}

void launch_wheel_bytes(const gbk::BatchParams &bp, uint32_t *out, cudaStream_t st)
{
    const uint32_t nw = (bp.nblk + 31) / 32;
    uint32_t blocks = (nw + 255) / 256;
    if (blocks > 65535) blocks = 65535;
    gbk::k_wheel_bytes<<<blocks, 256, 0, st>>>(bp, out);
}

}  // namespace gbh
