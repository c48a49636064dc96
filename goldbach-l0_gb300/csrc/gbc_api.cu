// gbc_api.cu -- the per-segment C ABI (include/gbc.h): context, tables,
// slots, batch planning, graph capture and replay, bounded-wait collect.
//
// Replaces the reference's Level Zero run driver plumbing
// (src/verifier.cpp:346-354 construction, 633-692 base primes, 853-1001
// buffer sizing, 1361-1440 table upload, 1741-2146 per-segment enqueue,
// 2402-2444 collect) for one CUDA device: nslots slots, each with its own
// stream, class-map buffer, first-bit table, result area and batch
// descriptor. A batch is planned on the host into the slot's pinned
// descriptor image; one host-to-device copy of it and a fixed sequence of
// persistent kernels (captured once per slot as a CUDA graph, then
// replayed) run the whole pipeline; it is collected later, so the host's
// work on batch k overlaps the GPU's work on batch k + 1.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "gbc_common.cuh"
#include "gbc_internal.h"

namespace {

constexpr uint32_t kGroupPrimes[gbk::kNumGroups][3] = {{7, 11, 13},  {17, 19, 23}, {29, 31, 1}, {37, 41, 1},
                                                       {43, 47, 1}, {53, 59, 1},   {61, 67, 1}};

uint64_t isqrt64(uint64_t n)
{
    uint64_t r = 0;
    for (int b = 31; b >= 0; --b) {
        const uint64_t t = r | (1ull << b);
        if (t <= n / t) r = t;
    }
    return r;
}

uint32_t inv_mod_small(uint32_t a, uint32_t m)  // a^-1 mod m, 0 if none
{
    int64_t t = 0, nt = 1, r = m, nr = a % m;
    while (nr) {
        const int64_t q = r / nr;
        int64_t x = t - q * nt;
        t = nt;
        nt = x;
        x = r - q * nr;
        r = nr;
        nr = x;
    }
    if (r != 1) return 0;
    if (t < 0) t += m;
    return uint32_t(t);
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

DescLayout::DescLayout(uint32_t nrun_cap, uint32_t nseg_cap)
{
    size_t o = align_up(sizeof(gbk::BatchHeader), 64);
    runs = o;
    o = align_up(o + size_t(nrun_cap) * sizeof(gbk::BatchParams), 64);
    segs = o;
    o = align_up(o + size_t(nseg_cap) * sizeof(gbk::SegParams), 64);
    tile_pref = o;
    o = align_up(o + size_t(nrun_cap + 1) * 4, 64);
    chk_pref = o;
    o = align_up(o + size_t(nseg_cap + 1) * 4, 64);
    ver_pref = o;
    o = align_up(o + size_t(nseg_cap + 1) * 4, 64);
    cnt_pref = o;
    o = align_up(o + size_t(nseg_cap + 1) * 4, 64);
    bytes = o;
}

gbk::BatchDesc DescLayout::device(const uint8_t *b) const
{
    gbk::BatchDesc d;
    d.h = reinterpret_cast<const gbk::BatchHeader *>(b);
    d.work = const_cast<uint32_t *>(d.h->work);
    d.runs = reinterpret_cast<const gbk::BatchParams *>(b + runs);
    d.segs = reinterpret_cast<const gbk::SegParams *>(b + segs);
    d.tile_pref = reinterpret_cast<const uint32_t *>(b + tile_pref);
    d.chk_pref = reinterpret_cast<const uint32_t *>(b + chk_pref);
    d.ver_pref = reinterpret_cast<const uint32_t *>(b + ver_pref);
    d.cnt_pref = reinterpret_cast<const uint32_t *>(b + cnt_pref);
    return d;
}

void DescImage::bind(uint8_t *b, const DescLayout &l)
{
    h = reinterpret_cast<gbk::BatchHeader *>(b);
    runs = reinterpret_cast<gbk::BatchParams *>(b + l.runs);
    segs = reinterpret_cast<gbk::SegParams *>(b + l.segs);
    tile_pref = reinterpret_cast<uint32_t *>(b + l.tile_pref);
    chk_pref = reinterpret_cast<uint32_t *>(b + l.chk_pref);
    ver_pref = reinterpret_cast<uint32_t *>(b + l.ver_pref);
    cnt_pref = reinterpret_cast<uint32_t *>(b + l.cnt_pref);
}

// The odd primes <= n (n < 2^32), by a segmented sieve on all host threads.
std::vector<uint32_t> gbh_odd_primes_upto(uint64_t n)
{
    std::vector<uint32_t> out;
    if (n < 3) return out;
    const uint64_t r = isqrt64(n);
    std::vector<uint8_t> comp(r + 1, 0);
    std::vector<uint32_t> small;
    for (uint64_t i = 2; i <= r; ++i)
        if (!comp[i]) {
            if (i & 1) small.push_back(uint32_t(i));
            for (uint64_t k = i * i; k <= r; k += i) comp[k] = 1;
        }
    const uint64_t nodd = (n - 1) / 2;  // odd numbers 3..n: index i <-> 2 i + 3
    const uint64_t blk = 1u << 21;
    const uint64_t nblk = (nodd + blk - 1) / blk;
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    if (nt > nblk) nt = unsigned(nblk ? nblk : 1);
    std::vector<std::vector<uint32_t>> parts(nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            std::vector<uint8_t> buf(blk);
            for (uint64_t b = nblk * t / nt; b < nblk * (t + 1) / nt; ++b) {
                const uint64_t i0 = b * blk, i1 = std::min(nodd, i0 + blk);
                std::fill(buf.begin(), buf.begin() + (i1 - i0), 1);
                const uint64_t v0 = 2 * i0 + 3, v1 = 2 * (i1 - 1) + 3;
                for (uint32_t p : small) {
                    const uint64_t pp = uint64_t(p) * p;
                    if (pp > v1) break;
                    uint64_t s = pp;
                    if (s < v0) {
                        s = (v0 + p - 1) / p * p;
                        if (!(s & 1)) s += p;
                    }
                    for (uint64_t v = s; v <= v1; v += 2ull * p) buf[(v - 3) / 2 - i0] = 0;
                }
                for (uint64_t i = i0; i < i1; ++i)
                    if (buf[i - i0]) parts[t].push_back(uint32_t(2 * i + 3));
            }
        });
    for (auto &x : th) x.join();
    size_t tot = 0;
    for (auto &p : parts) tot += p.size();
    out.reserve(tot);
    for (auto &p : parts) out.insert(out.end(), p.begin(), p.end());
    return out;
}

// The odd primes <= n, shared by the contexts of a process: the last list
// sieved is kept and a smaller bound takes a prefix of it.
std::vector<uint32_t> gbh_cached_primes(uint64_t n)
{
    static std::mutex mu;
    static std::shared_ptr<const std::vector<uint32_t>> last;
    static uint64_t last_n = 0;
    std::shared_ptr<const std::vector<uint32_t>> have;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (last && last_n >= n) have = last;
    }
    if (!have) {
        auto fresh = std::make_shared<const std::vector<uint32_t>>(gbh_odd_primes_upto(n));
        std::lock_guard<std::mutex> lk(mu);
        if (!last || last_n < n) {
            last = fresh;
            last_n = n;
        }
        have = fresh;
    }
    const auto end = std::upper_bound(have->begin(), have->end(), n);
    return std::vector<uint32_t>(have->begin(), end);
}

static int fail(gbc_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                    \
    do {                                                                                            \
        const cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                      \
            return fail(ctx, GBC_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
    } while (0)

// device allocation counted in the context's footprint
template <class T>
static cudaError_t dev_alloc(gbc_ctx *ctx, T **p, size_t bytes)
{
    const cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), bytes);
    if (e == cudaSuccess) ctx->device_bytes += bytes;
    return e;
}

extern "C" int gbc_candidates(uint16_t *out, int cap)
{
    std::vector<uint32_t> p = gbh_odd_primes_upto(GBC_MAX_CAND);
    const int n = int(p.size());
    for (int i = 0; i < n && i < cap; ++i) out[i] = uint16_t(p[i]);
    return n;
}

// class-array words of a run of nblk bits: 64 bits of slack for the
// checkers' window reads, rounded to 32 words (128-byte aligned maps)
static uint64_t run_wpc(uint64_t nblk) { return align_up((nblk + 64 + 31) / 32, 32); }

// Expected hit-list marks per class bit of a run whose q reach qmax: the
// density among integers of q = p m with p a prime in [p_hl, p_max] and m
// prime, 1 / L * ln(u1 (L - u0) / (u0 (L - u1))) (L = ln q, u = ln p; the
// sum over p of 1 / (p ln(q / p)) with the prime density 1 / ln), times
// 30 / 8 (every such q is coprime to 30).
static double hl_density(double qmax, double p_hl, double p_max)
{
    const double L = std::log(qmax), u0 = std::log(p_hl), u1 = std::log(std::min(p_max, std::sqrt(qmax)));
    if (u1 <= u0) return 0;
    return std::log(u1 * (L - u0) / (u0 * (L - u1))) / L * 30.0 / 8.0;
}

// Region bins of a binned batch: regions of 2^rlog bits of the virtual class
// array (at least 2^28: few bins per harvest CTA, so its shared-memory
// counters cover them), at most kHlMaxBins / 8 per class.
static void hl_regions(uint64_t nblk, uint32_t &rlog, uint32_t &nreg)
{
    rlog = 28;
    while (((nblk + (uint64_t(1) << rlog) - 1) >> rlog) > gbk::kHlMaxBins / 8) ++rlog;
    nreg = uint32_t((nblk + (uint64_t(1) << rlog) - 1) >> rlog);
}

// Offsets per (harvest CTA, bin): the expected marks of a whole region (not
// the batch's average over bins: its last region is cut short) + 45%, + 64,
// whole lines. marks_per_bit: marks per class bit. The margin covers the
// harvest CTAs' uneven shares: CTA c takes primes in blocks of 256, and the
// first blocks (the smallest primes, with the most marks) weigh most.
static uint32_t hl_quota(double marks_per_bit, uint64_t nblk, uint32_t rlog, uint32_t ctas)
{
    const double region = double(std::min<uint64_t>(nblk, uint64_t(1) << rlog));
    return uint32_t(align_up(size_t(1.45 * marks_per_bit * region / double(ctas)) + 64, 32));
}

// Offsets per tile bin: the expected marks of a tile + 15%, + 2048, whole
// lines (the density is that of the run's top, where it is highest).
static size_t tb_capacity(double marks_per_bit, uint32_t tile_bits)
{
    return align_up(size_t(1.15 * marks_per_bit * double(tile_bits)) + 2048, 32);
}

// tiles of a class array of `bits` bits
static uint32_t tiles_of(uint64_t bits, uint32_t tile_bits) { return uint32_t((bits + tile_bits - 1) / tile_bits); }

// the largest tile the persistent tile kernel takes: 224 KB of shared memory
constexpr uint32_t kMaxTileBits = 1835008;

// runs a batch's binned hit lists are sized for (the serving loop's
// batches hold 16, the windows leg's 64)
constexpr uint32_t kHlBinnedRuns = 64;

// overflow marks a binned batch may leave: 2% of a full batch's, at least 2^22
static uint32_t overflow_cap(double marks)
{
    return uint32_t(std::min(double(1u << 30), std::max(double(1u << 22), 0.02 * marks)));
}

// words past the end of the primes and their reciprocals: the tile kernel
// reads them four at a time
constexpr size_t kPrimePad = 4;

static int slot_alloc(gbc_ctx *ctx, Slot &s)
{
    const auto &cfg = ctx->cfg;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    for (auto &e : s.ev) CK(cudaEventCreate(&e));
    // max_batch full segments in one run, plus every further run's margin
    s.map_words = size_t(8) * ctx->wpc_cap + size_t(8) * cfg.max_runs * 448;
    CK(dev_alloc(ctx, &s.map, s.map_words * 4 + kMapPadBytes));
    CK(cudaMemset(s.map, 0, s.map_words * 4 + kMapPadBytes));
    s.xfirst_words = std::max<size_t>(size_t(8) * ctx->n_mid * cfg.max_runs, 1);
    CK(dev_alloc(ctx, &s.xfirst, s.xfirst_words * 4));
    CK(dev_alloc(ctx, &s.res, size_t(cfg.max_batch) * sizeof(gbc_segment_result)));
    CK(dev_alloc(ctx, &s.err, 4));
    if (cfg.want_pn) {
        s.pn_stride = cfg.segment_even / 2 + 1;
        CK(dev_alloc(ctx, &s.pn, size_t(cfg.max_batch) * s.pn_stride * 2));
    }
    // phase-A pending words: up to 1/16 of a segment's words (the plan
    // leaves ~1e-4 of the evens; an overflow fails the batch closed)
    s.pend_cap = uint32_t(std::max<uint64_t>(4096, (cfg.segment_even / 2 / 32 + 64) / 16));
    CK(dev_alloc(ctx, &s.pend, size_t(cfg.max_batch) * s.pend_cap * sizeof(uint2)));
    if (ctx->hl_on) {
        // binned hit lists for max_batch full segments at the density of the
        // context's top, in up to kHlBinnedRuns runs (each run's class array
        // starts a whole tile of the virtual array: a tile of slack per run;
        // batches of more runs, or that do not fit, clear their marks directly)
        const uint64_t nblk = uint64_t(ctx->wpc_cap) * 32 + uint64_t(kHlBinnedRuns) * ctx->tile_bits;
        uint32_t rlog, nreg;
        hl_regions(nblk, rlog, nreg);
        const uint32_t ctas = uint32_t(ctx->grids.sm) * uint32_t(ctx->grids.hitlist);
        const double marks = 8.0 * double(nblk) *
                             hl_density(double(cfg.limit) + 3, double(ctx->p_hl), double(ctx->primes.back()));
        s.hl_buf_words = size_t(ctas) * 8 * nreg * hl_quota(marks / (8.0 * double(nblk)), nblk, rlog, ctas);
        CK(dev_alloc(ctx, &s.hl_buf, std::max<size_t>(s.hl_buf_words, 1) * 4));
        CK(dev_alloc(ctx, &s.hl_cnt, size_t(ctas) * gbk::kHlMaxBins * 4));
        // tile bins: the tiles of a class array of wpc_cap words, and a tile per further run
        s.tb_cnt_words = size_t(8) * (tiles_of(uint64_t(ctx->wpc_cap) * 32, ctx->tile_bits) + kHlBinnedRuns);
        s.tb_buf_words = s.tb_cnt_words * tb_capacity(marks / (8.0 * double(nblk)), ctx->tile_bits);
        CK(dev_alloc(ctx, &s.tb_buf, std::max<size_t>(s.tb_buf_words, 1) * 4));
        CK(dev_alloc(ctx, &s.tb_cnt, std::max<size_t>(s.tb_cnt_words, 1) * 4));
        s.ovf_cap = overflow_cap(marks);
        CK(dev_alloc(ctx, &s.ovf_buf, size_t(s.ovf_cap) * sizeof(uint2)));
        CK(dev_alloc(ctx, &s.ovf_cnt, 4));
    }
    CK(cudaMallocHost(&s.desc_host, ctx->layout.bytes));
    CK(cudaMallocHost(&s.win_host, sizeof(gbk::BatchHeader) * cfg.max_batch));
    std::memset(s.desc_host, 0, ctx->layout.bytes);
    CK(dev_alloc(ctx, &s.desc_dev, ctx->layout.bytes));
    CK(cudaMemset(s.desc_dev, 0, ctx->layout.bytes));
    s.img.bind(s.desc_host, ctx->layout);
    s.dd = ctx->layout.device(s.desc_dev);
    return GBC_OK;
}

static void slot_free(Slot &s)
{
    if (s.st) cudaStreamSynchronize(s.st);
    if (s.exec) cudaGraphExecDestroy(s.exec);
    for (auto &e : s.ev)
        if (e) cudaEventDestroy(e);
    cudaFree(s.map);
    cudaFree(s.xfirst);
    cudaFree(s.res);
    cudaFree(s.err);
    cudaFree(s.pn);
    cudaFree(s.pend);
    cudaFree(s.desc_dev);
    cudaFree(s.hl_buf);
    cudaFree(s.hl_cnt);
    cudaFree(s.tb_buf);
    cudaFree(s.tb_cnt);
    cudaFree(s.ovf_buf);
    cudaFree(s.ovf_cnt);
    if (s.desc_host) cudaFreeHost(s.desc_host);
    if (s.win_host) cudaFreeHost(s.win_host);
    cudaFree(s.chk_map);
    cudaFree(s.chk_desc_dev);
    cudaFree(s.chk_count);
    if (s.chk_desc_host) cudaFreeHost(s.chk_desc_host);
    if (s.st) cudaStreamDestroy(s.st);
    s = Slot{};
}

extern "C" int gbc_create(const gbc_config *cfg_in, gbc_ctx **out)
{
    if (!out) return GBC_E_ARG;
    *out = nullptr;
    gbc_ctx *ctx = new (std::nothrow) gbc_ctx();
    if (!ctx) return GBC_E_ARG;
    gbc_config cfg{};
    if (cfg_in) cfg = *cfg_in;
    if (!cfg.limit) cfg.limit = 100000000ull;
    if (!cfg.segment_even) cfg.segment_even = GBC_DEFAULT_SEGMENT;
    if (cfg.segment_even & 1) cfg.segment_even += 1;
    if (!cfg.max_batch) cfg.max_batch = 8;
    if (!cfg.max_runs) cfg.max_runs = cfg.max_batch;
    if (!cfg.tile_log2) cfg.tile_log2 = 20;
    if (!cfg.p_mid) cfg.p_mid = 1u << 22;
    if (!cfg.mtab_max_gb) cfg.mtab_max_gb = 48;
    if (!cfg.nslots) cfg.nslots = 2;
    if (!cfg.sample_every) cfg.sample_every = 1;
    if (!cfg.plan_funnels) cfg.plan_funnels = 8;
    if (!cfg.ridge_min) cfg.ridge_min = GBC_TAIL_T;
    if (!cfg.launch_mode) cfg.launch_mode = 1;
    if (cfg.plan_funnels > gbk::kVerifyMaxFun) cfg.plan_funnels = gbk::kVerifyMaxFun;
    if (!cfg.verify_funnels) cfg.verify_funnels = 3;
    if (!cfg.hl_cap_pct || cfg.hl_cap_pct > 100) cfg.hl_cap_pct = 100;
    if (cfg.verify_funnels > cfg.plan_funnels) cfg.verify_funnels = cfg.plan_funnels;
    int rc = GBC_OK;
    if (cfg.limit > GBC_MAX_LIMIT || cfg.limit < 6) rc = fail(ctx, GBC_E_ARG, "limit outside [6, 2^64 - 2^40]");
    else if (cfg.segment_even < 1000 || cfg.segment_even > (1ull << 33))
        rc = fail(ctx, GBC_E_ARG, "segment_even outside [1000, 2^33]");
    else if (cfg.max_batch > 256) rc = fail(ctx, GBC_E_ARG, "max_batch above 256");
    else if (cfg.max_runs > cfg.max_batch) rc = fail(ctx, GBC_E_ARG, "max_runs above max_batch");
    else if (cfg.nslots < 2 || cfg.nslots > GBC_MAX_SLOTS) rc = fail(ctx, GBC_E_ARG, "nslots outside [2, 8]");
    else if (cfg.launch_mode > 3) rc = fail(ctx, GBC_E_ARG, "launch_mode outside [0, 3]");
    else if (cfg.tile_log2 < 14 || cfg.tile_log2 > 20) rc = fail(ctx, GBC_E_ARG, "tile_log2 outside [14, 20]");
    else if (cfg.tile_bits && (cfg.tile_bits % 4096 || cfg.tile_bits < (1u << 14) || cfg.tile_bits > kMaxTileBits))
        rc = fail(ctx, GBC_E_ARG, "tile_bits must be a multiple of 4096 in [2^14, 1835008]");
    else if (cfg.p_mid < 128) rc = fail(ctx, GBC_E_ARG, "p_mid below 128");
    else if (uint64_t(cfg.max_batch) * cfg.segment_even / 30 > (1ull << 31))
        rc = fail(ctx, GBC_E_ARG, "max_batch * segment_even / 30 must stay below 2^31 class bits");
    if (rc) {
        *out = ctx;  // let the caller read the message, then destroy
        return rc;
    }
    ctx->cfg = cfg;
    ctx->err.clear();
    cudaError_t e = cudaSetDevice(cfg.device);
    if (e != cudaSuccess) {
        *out = ctx;
        return fail(ctx, GBC_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    }
    int dev = cfg.device;
    cudaDeviceGetAttribute(&ctx->grids.sm, cudaDevAttrMultiProcessorCount, dev);
    if (ctx->grids.sm <= 0) ctx->grids.sm = 1;
    ctx->grids.max_seg = int(cfg.max_batch);

    // sieving primes: every odd prime <= floor(sqrt(limit + 3)) + 16, saturated below 2^32
    // (the reference's base_prime_bound, include/primes.hpp:222-225)
    const double rt = std::sqrt(double(cfg.limit + 3)) + 16.0;
    const uint64_t bound = rt >= 4294967295.0 ? 0xFFFFFFFFull : uint64_t(rt);
    ctx->primes = gbh_cached_primes(std::max<uint64_t>(bound, 127));
    const auto &pr = ctx->primes;
    ctx->i0 = uint32_t(std::lower_bound(pr.begin(), pr.end(), gbk::kFirstSievePrime) - pr.begin());
    ctx->n_mid = uint32_t(std::upper_bound(pr.begin(), pr.end(), cfg.p_mid) - pr.begin());
    ctx->tile_bits = cfg.tile_bits ? cfg.tile_bits : 1u << cfg.tile_log2;
    const uint32_t tb = ctx->tile_bits;
    // primes with at least 128 marks per tile: a warp per prime; above, a
    // thread per prime (measured on 128-segment batches at 4e18 with 2^20-bit
    // tiles: tb / 64 13.37 ms, tb / 128 13.03, tb / 256 13.55 per tile stage)
    ctx->i_warp = uint32_t(std::lower_bound(pr.begin(), pr.end(), std::max(tb / 128, 72u)) - pr.begin());
    if (ctx->i_warp > ctx->n_mid) ctx->i_warp = ctx->n_mid;
    std::vector<uint32_t> magic(ctx->n_mid);
    for (uint32_t i = 0; i < ctx->n_mid; ++i) magic[i] = uint32_t((1ull << 32) / pr[i]);
    // hit lists: every prime >= p_hl, p_hl above p_mid, above the cube root
    // of the largest q (the prime-multiplier rule needs p >= cbrt(q)), and
    // high enough that the table of multipliers m <= limit / p_hl fits the
    // HBM budget
    {
        uint64_t c = uint64_t(std::cbrt(double(cfg.limit + 3))) + 2;
        while (c * c * c < cfg.limit + 3) ++c;
        const uint64_t budget_m = uint64_t(cfg.mtab_max_gb) * 1000000000ull * 30;
        // (a little under the budget: the table is rounded up to 32-byte words)
        const uint64_t by_budget = (cfg.limit + 3) / (budget_m - budget_m / 1024) + 1;
        ctx->p_hl = std::max<uint64_t>({uint64_t(cfg.p_mid) + 1, c, by_budget});
        ctx->n_hl = uint32_t(std::lower_bound(pr.begin(), pr.end(), ctx->p_hl) - pr.begin());
        if (ctx->n_hl < ctx->n_mid) ctx->n_hl = ctx->n_mid;
        const bool wide = double(cfg.max_batch) * double(cfg.segment_even) >= 1e9;
        ctx->hl_on = cfg.hl_mode == 1 || (cfg.hl_mode == 0 && wide);
        if (ctx->n_hl >= pr.size()) ctx->hl_on = false;
    }

    // pattern groups (primes 7..67): canonical bit y = (y mod P coprime to P)
    std::vector<uint32_t> pat;
    for (int g = 0; g < gbk::kNumGroups; ++g) {
        uint32_t P = 1;
        for (int j = 0; j < 3; ++j) P *= kGroupPrimes[g][j];
        const uint32_t words = (P + 64 + 31) / 32 + 1;
        ctx->gi.P[g] = P;
        ctx->gi.off[g] = uint32_t(pat.size());
        ctx->gi.inv30[g] = inv_mod_small(30 % P, P);
        for (uint32_t wd = 0; wd < words; ++wd) {
            uint32_t v = 0;
            for (uint32_t b = 0; b < 32; ++b) {
                const uint32_t y = (wd * 32 + b) % P;
                bool keep = true;
                for (int j = 0; j < 3; ++j)
                    if (kGroupPrimes[g][j] > 1 && y % kGroupPrimes[g][j] == 0) keep = false;
                if (keep) v |= 1u << b;
            }
            pat.push_back(v);
        }
    }
    ctx->gi.words = uint32_t(pat.size());
    // the large primes' multiplier wheel mod 1001 = 7 * 11 * 13: per residue
    // x the rank of the first unit >= x (wrapping) | its distance << 10, the
    // gaps between consecutive units, the inverses mod 1001, the inverses mod
    // each of 17..43 (k_large)
    std::vector<uint16_t> wheel;
    {
        std::vector<uint32_t> units;
        for (uint32_t x = 0; x < gbk::kWheelM; ++x)
            if (x % 7 && x % 11 && x % 13) units.push_back(x);
        for (uint32_t x = 0; x < gbk::kWheelM; ++x) {
            const auto it = std::lower_bound(units.begin(), units.end(), x);
            const uint32_t rank = it == units.end() ? 0u : uint32_t(it - units.begin());
            const uint32_t dist = it == units.end() ? units[0] + gbk::kWheelM - x : *it - x;
            wheel.push_back(uint16_t(rank | dist << 10));
        }
        for (size_t r = 0; r < units.size(); ++r)
            wheel.push_back(uint16_t(r + 1 < units.size() ? units[r + 1] - units[r] : units[0] + gbk::kWheelM - units[r]));
        for (uint32_t x = 0; x < gbk::kWheelM; ++x) wheel.push_back(uint16_t(inv_mod_small(x, gbk::kWheelM)));
        for (uint32_t f : {17u, 19u, 23u, 29u, 31u, 37u, 41u, 43u})
            for (uint32_t x = 0; x < f; ++x) wheel.push_back(uint16_t(inv_mod_small(x, f)));
        if (units.size() != 720 || wheel.size() != gbk::kWheelTabWords) {
            *out = ctx;
            return fail(ctx, GBC_E_ARG, "wheel table size");
        }
    }
    // candidates and their per-class lists (useful: r - p coprime to 30)
    std::vector<uint32_t> c32 = gbh_odd_primes_upto(GBC_MAX_CAND);
    if (c32.size() != GBC_NCAND) {
        *out = ctx;
        return fail(ctx, GBC_E_ARG, "candidate count mismatch");
    }
    std::vector<uint16_t> cand(c32.begin(), c32.end()), list;
    for (int cr = 0; cr < GBC_NCLASS; ++cr) {
        ctx->ct.off[cr] = uint32_t(list.size());
        for (int i = 0; i < GBC_NCAND; ++i) {
            const uint32_t u = (2u * cr + 30 - cand[i] % 30) % 30;
            if (gbk::class_of(u) < 8) list.push_back(uint16_t(i));
        }
        ctx->ct.cnt[cr] = uint32_t(list.size()) - ctx->ct.off[cr];
        if (cfg.test_flags & GBC_TEST_RETRY_LIMIT) ctx->ct.cnt[cr] = std::min<uint32_t>(ctx->ct.cnt[cr], 1);
    }
    // verify plan (the reference's make_plan30, include/check30.hpp:88-174,
    // with our own greedy order): per class, the useful candidates below
    // GBC_TAIL_T in ascending order, each uncovered one p opening a funnel
    // with every uncovered prime of its residue among p + 30, ..., p + 930
    // (the 32 positions one 64-bit window read covers: member p + 30 d is
    // the top member's window shifted by its distance), plan_funnels
    // funnels, then ordered by member count; the rest lists hold every
    // useful candidate no funnel tests, ascending, for the exact
    // continuation.
    std::vector<uint2> fun;
    std::vector<uint16_t> rest;
    {
        std::vector<int> cidx(GBC_MAX_CAND + 1, -1);
        for (int i = 0; i < GBC_NCAND; ++i) cidx[cand[i]] = i;
        for (int cr = 0; cr < GBC_NCLASS; ++cr) {
            std::vector<char> covered(GBC_NCAND, 0);
            ctx->vt.fun_off[cr] = uint32_t(fun.size());
            const uint32_t b = ctx->ct.off[cr], e = b + ctx->ct.cnt[cr];
            for (uint32_t li = b; li < e; ++li) {
                const int i = list[li];
                if (fun.size() - ctx->vt.fun_off[cr] >= cfg.plan_funnels || cand[i] >= GBC_TAIL_T) break;
                if (covered[i]) continue;
                uint32_t mask = 1;
                covered[i] = 1;
                for (uint32_t d = 1; d < 32; ++d) {
                    const uint32_t q = cand[i] + 30 * d;
                    if (q >= GBC_TAIL_T || q > GBC_MAX_CAND) break;
                    if (cidx[q] < 0 || covered[cidx[q]]) continue;
                    covered[cidx[q]] = 1;
                    mask |= 1u << d;
                }
                fun.push_back(make_uint2(uint32_t(i), mask));
            }
            // every useful candidate resolves the same share of the evens
            // left (q is prime with probability 3.75 / ln q for any of
            // them), so the funnels with the most members go first
            std::stable_sort(fun.begin() + ctx->vt.fun_off[cr], fun.end(),
                             [](const uint2 &a, const uint2 &b) { return __builtin_popcount(a.y) > __builtin_popcount(b.y); });
            ctx->vt.fun_cnt[cr] = uint32_t(fun.size()) - ctx->vt.fun_off[cr];
            ctx->vt.rest_off[cr] = uint32_t(rest.size());
            for (uint32_t li = b; li < e; ++li)
                if (!covered[list[li]]) rest.push_back(list[li]);
            ctx->vt.rest_cnt[cr] = uint32_t(rest.size()) - ctx->vt.rest_off[cr];
        }
    }

    // one run of max_batch full segments plus the 9781 + 3 margin
    const uint64_t span = uint64_t(cfg.max_batch) * cfg.segment_even + GBC_MAX_CAND + 3 + 64;
    const uint64_t nblk_cap = span / 30 + 4;
    ctx->wpc_cap = uint32_t(std::max<uint64_t>(run_wpc(nblk_cap), align_up(run_wpc(nblk_cap), tb / 32)));
    ctx->layout = DescLayout(cfg.max_runs, cfg.max_batch);

    *out = ctx;
    if (!gbh::tile_attributes(ctx->tile_bits, cfg.tile_log2, ctx->gi, cfg.device, &ctx->tile_stage))
        return fail(ctx, GBC_E_ARG, "tile_bits: the tile does not fit the device's shared memory");
    gbh::query_check_grids(ctx->grids);
    gbh::query_count_grids(ctx->grids);
    gbh::query_sieve_grids(ctx->grids);
    CK(dev_alloc(ctx, &ctx->d_primes, (pr.size() + kPrimePad) * 4));
    CK(cudaMemcpy(ctx->d_primes, pr.data(), pr.size() * 4, cudaMemcpyHostToDevice));
    CK(dev_alloc(ctx, &ctx->d_magic, (magic.size() + kPrimePad) * 4));
    if (!magic.empty()) CK(cudaMemcpy(ctx->d_magic, magic.data(), magic.size() * 4, cudaMemcpyHostToDevice));
    CK(dev_alloc(ctx, &ctx->d_pat, pat.size() * 4));
    CK(cudaMemcpy(ctx->d_pat, pat.data(), pat.size() * 4, cudaMemcpyHostToDevice));
    CK(dev_alloc(ctx, &ctx->d_wheel, wheel.size() * 2));
    CK(cudaMemcpy(ctx->d_wheel, wheel.data(), wheel.size() * 2, cudaMemcpyHostToDevice));
    // the large primes from n_mid on, one byte each: (p_i - p_(i-1)) / 2, 0
    // at the start of each group of kPackGroup, whose first prime is kept
    // whole (pack_large_primes, src/host_math.cpp:187-209)
    {
        const size_t n = pr.size() > ctx->n_mid ? pr.size() - ctx->n_mid : 0;
        const size_t groups = std::max<size_t>((n + gbk::kPackGroup - 1) / gbk::kPackGroup, 1);
        std::vector<uint8_t> gap(groups * gbk::kPackGroup, 0);
        std::vector<uint32_t> gbase(groups, 0);
        for (size_t i = 0; i < n; ++i) {
            const uint32_t p = pr[ctx->n_mid + i];
            if (i % gbk::kPackGroup == 0) {
                gbase[i / gbk::kPackGroup] = p;
                continue;
            }
            const uint32_t g = p - pr[ctx->n_mid + i - 1];
            if ((g & 1) || g / 2 > 255) return fail(ctx, GBC_E_ARG, "a prime gap does not fit the packed stream");
            gap[i] = uint8_t(g / 2);
        }
        CK(dev_alloc(ctx, &ctx->d_pk_gap, gap.size()));
        CK(cudaMemcpy(ctx->d_pk_gap, gap.data(), gap.size(), cudaMemcpyHostToDevice));
        CK(dev_alloc(ctx, &ctx->d_pk_base, gbase.size() * 4));
        CK(cudaMemcpy(ctx->d_pk_base, gbase.data(), gbase.size() * 4, cudaMemcpyHostToDevice));
    }
    CK(dev_alloc(ctx, &ctx->d_cand, cand.size() * 2));
    CK(cudaMemcpy(ctx->d_cand, cand.data(), cand.size() * 2, cudaMemcpyHostToDevice));
    CK(dev_alloc(ctx, &ctx->d_list, list.size() * 2));
    CK(cudaMemcpy(ctx->d_list, list.data(), list.size() * 2, cudaMemcpyHostToDevice));
    ctx->ct.cand = ctx->d_cand;
    ctx->ct.list = ctx->d_list;
    ctx->ct.ridge_min = cfg.ridge_min;
    CK(dev_alloc(ctx, &ctx->d_fun, std::max<size_t>(fun.size(), 1) * sizeof(uint2)));
    if (!fun.empty()) CK(cudaMemcpy(ctx->d_fun, fun.data(), fun.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    // member pairs of each funnel: in shift space (member p0 + 30 d at shift
    // dm - d below the top member), pairs {a, a + delta} inside the members,
    // each tested by one shift of the window ORed with itself shifted by
    // delta; the delta with the fewest shifts (+ 4 for the OR) or none
    {
        std::vector<uint2> pairs(std::max<size_t>(fun.size(), 1), make_uint2(0u, 0u));
        for (size_t f = 0; f < fun.size(); ++f) {
            const uint32_t y = fun[f].y;
            const int dm = 31 - __builtin_clz(y);
            uint32_t S = 0;
            for (int d = 0; d <= dm; ++d)
                if (y >> d & 1u) S |= 1u << (dm - d);
            // costs in half ALU operations: a member 3 (a funnel shift and
            // half a three-input OR), the OR of the window with its shift 8
            int best_cost = 3 * __builtin_popcount(S), best_delta = 0;
            uint32_t best_a = 0;
            for (int delta = 1; delta < 32; ++delta) {
                uint32_t used = 0, A = 0;
                for (int a = 0; a + delta < 32; ++a)
                    if ((S >> a & 1u) && (S >> (a + delta) & 1u) && !(used >> a & 1u) && !(used >> (a + delta) & 1u)) {
                        A |= 1u << a;
                        used |= (1u << a) | (1u << (a + delta));
                    }
                const uint32_t R = S & ~used;
                const int cost = 8 + 3 * (__builtin_popcount(A) + __builtin_popcount(R));
                const int groups = (__builtin_popcount(A) + 3) / 4 + (__builtin_popcount(R) + 3) / 4;
                if (A && cost < best_cost && groups <= int(gbk::kVerifyMaxGroups)) {
                    best_cost = cost;
                    best_delta = delta;
                    best_a = A;
                }
            }
            pairs[f] = make_uint2(uint32_t(best_delta), best_a);
        }
        CK(dev_alloc(ctx, &ctx->d_fpair, pairs.size() * sizeof(uint2)));
        CK(cudaMemcpy(ctx->d_fpair, pairs.data(), pairs.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    }
    CK(dev_alloc(ctx, &ctx->d_rest, std::max<size_t>(rest.size(), 1) * 2));
    if (!rest.empty()) CK(cudaMemcpy(ctx->d_rest, rest.data(), rest.size() * 2, cudaMemcpyHostToDevice));
    ctx->vt.cand = ctx->d_cand;
    ctx->vt.fun = ctx->d_fun;
    ctx->vt.fpair = ctx->d_fpair;
    ctx->vt.rest = ctx->d_rest;
    ctx->vt.ridge_min = cfg.ridge_min;
    ctx->vt.f1 = cfg.verify_funnels;
    ctx->vt.spin0 = (cfg.test_flags & GBC_TEST_STAGING_WAIT) ? 0u : gbk::kStageSpin;
    ctx->slot.resize(cfg.nslots);
    for (auto &s : ctx->slot)
        if (int r = slot_alloc(ctx, s)) return r;
    CK(cudaDeviceSynchronize());
    return GBC_OK;
}

extern "C" void gbc_destroy(gbc_ctx *ctx)
{
    if (!ctx) return;
    if (ctx->outputs && ctx->outputs_del) ctx->outputs_del(ctx->outputs);
    if (ctx->stats && ctx->stats_del) ctx->stats_del(ctx->stats);
    for (auto &s : ctx->slot) slot_free(s);
    cudaFree(ctx->d_fun);
    cudaFree(ctx->d_fpair);
    cudaFree(ctx->d_rest);
    cudaFree(ctx->mtab);
    cudaFree(ctx->d_primes);
    cudaFree(ctx->d_magic);
    cudaFree(ctx->d_pat);
    cudaFree(ctx->d_wheel);
    cudaFree(ctx->d_pk_gap);
    cudaFree(ctx->d_pk_base);
    cudaFree(ctx->d_cand);
    cudaFree(ctx->d_list);
    delete ctx;
}

// the run driver's (gb_run.cpp) failure text for gbc_last_error
void gbh_set_outputs(gbc_ctx *ctx, void *p, void (*del)(void *))
{
    if (ctx->outputs && ctx->outputs_del) ctx->outputs_del(ctx->outputs);
    ctx->outputs = p;
    ctx->outputs_del = del;
}

void *gbh_outputs(gbc_ctx *ctx) { return ctx ? ctx->outputs : nullptr; }

// the campaign statistics of runs on the context (gb_run.cpp)
void gbh_set_stats(gbc_ctx *ctx, void *p, void (*del)(void *), bool gaps)
{
    if (ctx->stats && ctx->stats_del) ctx->stats_del(ctx->stats);
    ctx->stats = p;
    ctx->stats_del = del;
    ctx->stats_gaps = gaps;
}

void *gbh_stats(gbc_ctx *ctx, bool *gaps)
{
    if (gaps) *gaps = ctx && ctx->stats_gaps;
    return ctx ? ctx->stats : nullptr;
}

void gbh_set_error(gbc_ctx *ctx, const char *msg)
{
    if (ctx) ctx->err = msg;
}

extern "C" const char *gbc_last_error(const gbc_ctx *ctx)
{
    if (!ctx) return "no context";
    return ctx->err.c_str();
}

extern "C" int gbc_get_config(const gbc_ctx *ctx, gbc_config *out)
{
    if (!ctx || !out) return GBC_E_ARG;
    *out = ctx->cfg;
    return GBC_OK;
}

static bool bad_slot(const gbc_ctx *ctx, int slot) { return !ctx || slot < 0 || slot >= int(ctx->slot.size()); }

extern "C" void *gbc_stream(gbc_ctx *ctx, int slot)
{
    if (bad_slot(ctx, slot)) return nullptr;
    return ctx->slot[slot].st;
}

extern "C" uint64_t gbc_launch_count(const gbc_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" int gbc_get_stats(const gbc_ctx *ctx, gbc_ctx_stats *out)
{
    if (!ctx || !out) return GBC_E_ARG;
    out->launches = ctx->launches;
    out->batches = ctx->batches;
    out->graph_replays = ctx->graph_replays;
    out->selfchecks = ctx->selfchecks;
    out->mtab_builds = ctx->mtab_builds;
    out->mtab_bytes = ctx->mtab_bytes;
    out->mtab_build_ms = ctx->mtab_build_ms;
    out->device_bytes = ctx->device_bytes;
    out->p_hl = ctx->hl_on ? ctx->p_hl : 0;
    out->sm_count = uint32_t(ctx->grids.sm);
    out->hl_overflow = ctx->hl_overflow;
    return GBC_OK;
}

// the run base's residues the large-prime kernel's wheel and skip lanes start from
static void set_residues(gbk::BatchParams &bp)
{
    bp.bm1 = uint32_t(bp.base % gbk::kWheelM);
    const uint32_t f[8] = {17, 19, 23, 29, 31, 37, 41, 43};
    for (int j = 0; j < 8; ++j) bp.bres[j] = uint8_t(bp.base % f[j]);
}

// One run (class map) of a batch: geometry, primes that reach it, and the
// shared tables (the reference's segment_geometry / class_geometry,
// src/host_math.cpp:13-78, for one map per run).
static void plan_run(const gbc_ctx *ctx, gbk::BatchParams &bp, uint64_t s0, uint64_t sN)
{
    const auto &pr = ctx->primes;
    const uint64_t qlo = s0 > GBC_MAX_CAND + 30 ? s0 - GBC_MAX_CAND : 0;
    bp.base = qlo / 30 * 30;
    bp.qmax = sN + 3;
    const uint64_t nblk = (bp.qmax - bp.base) / 30 + 1;
    bp.nblk = uint32_t(nblk);
    bp.wpc = uint32_t(run_wpc(nblk));
    bp.tiles_pc = tiles_of(uint64_t(bp.wpc) * 32, ctx->tile_bits);
    bp.tb_vt0 = 0;
    bp.tb_tiles = bp.tiles_pc;
    bp.tile_log2 = ctx->cfg.tile_log2;
    bp.tile_bits = ctx->tile_bits;
    bp.tile_rcp = uint32_t(((uint64_t(1) << 32) + ctx->tile_bits - 1) / ctx->tile_bits);
    bp.primes = ctx->d_primes;
    bp.magic = ctx->d_magic;
    bp.pat = ctx->d_pat;
    bp.wheel = ctx->d_wheel;
    bp.pk_gap = ctx->d_pk_gap;
    bp.pk_base = ctx->d_pk_base;
    bp.pk_i0 = ctx->n_mid;
    const uint64_t root = isqrt64(bp.qmax);
    bp.n_all = uint32_t(std::upper_bound(pr.begin(), pr.end(), root) - pr.begin());
    bp.i0 = std::min(ctx->i0, bp.n_all);
    bp.n_mid = std::max(std::min(ctx->n_mid, bp.n_all), bp.i0);
    bp.i_warp = std::min(std::max(ctx->i_warp, bp.i0), bp.n_mid);
    bp.n_hl = ctx->hl_on ? std::min(std::max(ctx->n_hl, bp.n_mid), bp.n_all) : bp.n_all;
    set_residues(bp);
}

// Fills the descriptor prefix arrays and header counts from its runs and
// segments (img.h->nrun, nseg, runs and segs already set).
static void finish_desc(const gbc_ctx *ctx, DescImage &img)
{
    gbk::BatchHeader &h = *img.h;
    const uint32_t nrun = h.nrun, nseg = h.nseg;
    h.tile_items = 0;
    h.n_mid_max = 0;
    h.n_mid_min = UINT32_MAX;
    h.n_hl_max = 0;
    h.n_hl_min = UINT32_MAX;
    h.n_all_max = 0;
    for (uint32_t r = 0; r < nrun; ++r) {
        const gbk::BatchParams &bp = img.runs[r];
        img.tile_pref[r] = h.tile_items;
        h.tile_items += 8 * bp.tiles_pc;
        h.n_mid_max = std::max(h.n_mid_max, bp.n_mid);
        h.n_mid_min = std::min(h.n_mid_min, bp.n_mid);
        h.n_hl_max = std::max(h.n_hl_max, bp.n_hl);
        h.n_hl_min = std::min(h.n_hl_min, bp.n_hl);
        h.n_all_max = std::max(h.n_all_max, bp.n_all);
    }
    img.tile_pref[nrun] = h.tile_items;
    if (!nrun) h.n_mid_min = h.n_hl_min = 0;
    h.chk_vb = h.ver_vb = h.cnt_vb = h.nlow = 0;
    for (uint32_t i = 0; i < nseg; ++i) {
        gbk::SegParams &sp = img.segs[i];
        img.chk_pref[i] = h.chk_vb;
        img.ver_pref[i] = h.ver_vb;
        img.cnt_pref[i] = h.cnt_vb;
        const uint64_t evens = (sp.seg_end - sp.seg_start) / 2 + 1;
        sp.vbx = gbh::check_vbx(evens, ctx->grids.sm);
        if (sp.low) ++h.nlow;
        else if (sp.sampled) h.chk_vb += GBC_NCLASS * sp.vbx;
        else h.ver_vb += GBC_NCLASS * sp.vbx;
        h.cnt_vb += gbh::count_ranges(img.runs[sp.run].base, sp, sp.cr);
    }
    img.chk_pref[nseg] = h.chk_vb;
    img.ver_pref[nseg] = h.ver_vb;
    img.cnt_pref[nseg] = h.cnt_vb;
    h.seg0 = 0;  // the whole batch
    h.win_b0 = 0;
    h.win_b1 = UINT32_MAX;
}

// The plain form's per-segment headers (launch mode 3, a one-run batch):
// segment i's tiles (those of its q range [hash_lo, hash_hi] and 64 bits of
// the checkers' slack; a tile shared with a neighbour is sieved again, the
// same bits), its virtual CTAs of the checkers and the count kernel, and the
// class bits of those tiles for the large primes and the overflow marks.
static void plain_windows(const gbc_ctx *ctx, Slot &s)
{
    const DescImage &img = s.img;
    const gbk::BatchParams &bp = img.runs[0];
    const uint32_t tb = ctx->tile_bits, nseg = img.h->nseg;
    for (uint32_t i = 0; i < nseg; ++i) {
        const gbk::SegParams &sp = img.segs[i];
        gbk::BatchHeader h = *img.h;
        const uint64_t lo = sp.hash_lo > bp.base ? (sp.hash_lo - bp.base) / 30 : 0;
        const uint64_t hi = (sp.hash_hi - bp.base) / 30 + 64;
        const uint32_t ti0 = uint32_t(lo / tb), ti1 = uint32_t(std::min<uint64_t>(hi / tb, bp.tiles_pc - 1));
        h.tile_items = 8 * (ti1 + 1);
        h.work[gbk::kWorkTile] = 8 * ti0;
        h.chk_vb = img.chk_pref[i + 1];
        h.work[gbk::kWorkCheck] = img.chk_pref[i];
        h.ver_vb = img.ver_pref[i + 1];
        h.work[gbk::kWorkVerify] = img.ver_pref[i];
        h.cnt_vb = img.cnt_pref[i + 1];
        h.work[gbk::kWorkCount] = img.cnt_pref[i];
        h.nseg = i + 1;
        h.seg0 = i;
        h.win_b0 = ti0 * tb;
        h.win_b1 = uint32_t(std::min<uint64_t>(uint64_t(ti1 + 1) * tb, uint64_t(bp.wpc) * 32));
        s.win_host[i] = h;
    }
}

// Plans a batch into the slot's descriptor image: runs, their maps in the
// slot's buffer, segments (the reference's prepare_segment_tables, seg30 and
// count30_limits, src/verifier.cpp:1741-1767, include/check30.hpp:196-210,
// include/gstats.hpp:272-296).
static int plan_batch(gbc_ctx *ctx, Slot &s, const uint64_t *b, const uint32_t *fl, const uint64_t *lim, int nseg)
{
    const auto &cfg = ctx->cfg;
    if (nseg < 1 || uint32_t(nseg) > cfg.max_batch) return fail(ctx, GBC_E_ARG, "nseg outside [1, max_batch]");
    for (int i = 0; i < nseg; ++i) {
        const uint64_t a = b[2 * i], e = b[2 * i + 1], l = lim[i];
        if (l > cfg.limit || l & 1) return fail(ctx, GBC_E_ARG, "limit odd or above the context's limit");
        if ((a | e) & 1 || a < 4 || e < a || e > l)
            return fail(ctx, GBC_E_ARG, "segment bounds must be even with 4 <= start <= end <= limit");
        if (e - a > cfg.segment_even) return fail(ctx, GBC_E_ARG, "segment longer than segment_even");
    }
    DescImage &img = s.img;
    uint32_t nrun = 0;
    uint64_t map_off = 0, xf_off = 0;
    for (int i = 0; i < nseg;) {
        int j = i + 1;
        while (j < nseg && b[2 * j] == b[2 * j - 1] + 2) ++j;
        if (nrun == cfg.max_runs) return fail(ctx, GBC_E_ARG, "more runs than max_runs");
        gbk::BatchParams &bp = img.runs[nrun];
        bp = gbk::BatchParams{};
        plan_run(ctx, bp, b[2 * i], b[2 * j - 1]);
        const uint64_t words = uint64_t(8) * bp.wpc;
        if (map_off + words > s.map_words) return fail(ctx, GBC_E_ARG, "batch wider than the slot's class map");
        bp.map = s.map + map_off;
        bp.xfirst = s.xfirst + xf_off;
        bp.err = s.err;
        bp.spin0 = (ctx->cfg.test_flags & GBC_TEST_STAGING_WAIT) ? 0u : gbk::kStageSpin;
        map_off += words;
        xf_off += uint64_t(8) * bp.n_mid;
        for (int k = i; k < j; ++k) img.segs[k].run = nrun;
        ++nrun;
        i = j;
    }
    for (int i = 0; i < nseg; ++i) {
        gbk::SegParams &sp = img.segs[i];
        const uint32_t run = sp.run;
        sp = gbk::SegParams{};
        sp.run = run;
        const uint64_t limit = lim[i];
        sp.seg_start = b[2 * i];
        sp.seg_end = b[2 * i + 1];
        sp.flags = fl ? fl[i] : 0;
        sp.low = sp.seg_start < GBC_MAX_CAND + 7 ? 1 : 0;
        const bool last = sp.seg_end == limit;
        sp.cnt_lo = sp.seg_start + 1;
        sp.cnt_hi = last ? limit - 1 : sp.seg_end + 1;
        sp.twin_hi = std::min(sp.cnt_hi, limit >= 3 ? limit - 3 : 0);
        sp.hash_lo = sp.seg_start > GBC_MAX_CAND + 1 ? sp.seg_start - GBC_MAX_CAND : 1;
        sp.hash_hi = sp.seg_end + 3;
        sp.res = s.res + i;
        sp.pn = s.pn ? s.pn + size_t(i) * s.pn_stride : nullptr;
        // the low segment and callers that want p(n) of every even take the exact checker
        sp.sampled = (sp.flags & GBC_SEG_VERIFY) && !sp.low && !sp.pn ? 0 : 1;
        sp.pend = s.pend + size_t(i) * s.pend_cap;
        sp.pend_cap = s.pend_cap;
    }
    img.h->nrun = nrun;
    img.h->nseg = uint32_t(nseg);
    // a batch with hit-listed runs: marks binned by region of the virtual
    // class array (the runs end to end, each from a whole tile), then by tile
    bool any_hl = false;
    for (uint32_t r = 0; r < nrun; ++r) any_hl |= img.runs[r].n_hl < img.runs[r].n_all;
    if (s.hl_buf && any_hl) {
        uint64_t vt = 0;        // virtual tiles per class
        double density = 0.0;   // marks per class bit, the densest run's
        for (uint32_t r = 0; r < nrun; ++r) {
            const gbk::BatchParams &bp = img.runs[r];
            vt += bp.tiles_pc;
            if (bp.n_hl < bp.n_all)
                density = std::max(density, hl_density(double(bp.qmax), double(ctx->primes[bp.n_hl]),
                                                       double(ctx->primes[bp.n_all - 1])));
        }
        const uint64_t vbits = vt * ctx->tile_bits;
        uint32_t rlog, nreg;
        hl_regions(vbits, rlog, nreg);
        const uint32_t ctas = uint32_t(ctx->grids.sm) * uint32_t(ctx->grids.hitlist), nbin = 8 * nreg;
        const uint32_t pct = ctx->cfg.hl_cap_pct;
        const uint32_t quota = uint32_t(
            std::max<size_t>(32, align_up(size_t(hl_quota(density, vbits, rlog, ctas)) * pct / 100, 32)));
        const size_t tiles = size_t(8) * vt,
                     tcap = std::max<size_t>(32, align_up(tb_capacity(density, ctx->tile_bits) * pct / 100, 32));
        // k_binsort sorts a region's offsets by tile in shared memory: at
        // most kSortMaxTiles tiles meet a region; virtual bits stay below
        // 2^31 (tile_of)
        const bool tb_fit = tiles_of(uint64_t(1) << rlog, ctx->tile_bits) + 1 <= gbk::kSortMaxTiles &&
                            tiles <= s.tb_cnt_words && tiles * tcap <= s.tb_buf_words && tcap < (1ull << 31) &&
                            vbits < (uint64_t(1) << 31) && nbin <= gbk::kHlMaxBins;
        if (size_t(ctas) * nbin * quota <= s.hl_buf_words && tb_fit) {
            uint32_t vt0 = 0;
            for (uint32_t r = 0; r < nrun; ++r) {
                gbk::BatchParams &bp = img.runs[r];
                bp.hl_buf = s.hl_buf;
                bp.hl_cnt = s.hl_cnt;
                bp.hl_quota = quota;
                bp.hl_rlog = rlog;
                bp.hl_nreg = nreg;
                bp.hl_ctas = ctas;
                bp.tb_buf = s.tb_buf;
                bp.tb_cnt = s.tb_cnt;
                bp.tb_cap = uint32_t(tcap);
                bp.tb_vt0 = vt0;
                bp.tb_tiles = uint32_t(vt);
                bp.ovf_buf = s.ovf_buf;
                bp.ovf_cnt = s.ovf_cnt;
                bp.ovf_cap = s.ovf_cap;
                vt0 += bp.tiles_pc;
            }
        }
    }
    finish_desc(ctx, img);
    return GBC_OK;
}

// Makes the prime-multiplier table cover the multipliers [need0, need1]:
// the primes m of the range, one byte per block of 30 (bit k <-> m = m0 +
// 30 i + u_k), sieved by the batch kernels themselves in chunks and
// rewritten to bytes (the reference's mt_build, src/verifier.cpp:1444-1508,
// goldbach.cl:3181-3242). Rebuilt only when a batch needs multipliers
// outside it; every slot is drained first (they read the table).
static int ensure_mtab(gbc_ctx *ctx, uint64_t need0, uint64_t need1)
{
    if (ctx->mtab && ctx->mtab_m0 <= need0 && need1 <= ctx->mtab_m1) return GBC_OK;
    const auto t0 = std::chrono::steady_clock::now();
    for (auto &s : ctx->slot) CK(cudaStreamSynchronize(s.st));
    if (ctx->mtab) {
        // keep covering what the old table covered
        need0 = std::min(need0, ctx->mtab_m0);
        need1 = std::max(need1, ctx->mtab_m1);
    }
    const uint64_t cap_bytes = uint64_t(ctx->cfg.mtab_max_gb) * 1000000000ull;
    // headroom for the batches that follow (a slice moves need1 by ~1e-4 per batch)
    uint64_t lo = need0 - need0 / 64, hi = need1 + need1 / 64 + (1u << 20);
    if ((hi - lo) / 30 + 1 > cap_bytes) {
        lo = need0;
        hi = need1;
    }
    lo = lo / 30 * 30;
    const uint64_t nbytes = ((hi - lo) / 30 + 1 + 31) / 32 * 32;
    if (nbytes > cap_bytes) return fail(ctx, GBC_E_ARG, "prime-multiplier table above its HBM budget");
    hi = lo + 30 * nbytes - 1;
    if (ctx->mtab) {
        cudaFree(ctx->mtab);
        ctx->device_bytes -= ctx->mtab_bytes + 64;
    }
    ctx->mtab = nullptr;
    ctx->mtab_bytes = 0;
    CK(dev_alloc(ctx, &ctx->mtab, nbytes + 64));
    ctx->mtab_bytes = nbytes;
    // sieve [lo, hi] in chunks through a temporary class map, each chunk a
    // one-run batch of its own descriptor (all uploaded before the first launch)
    const uint32_t tb = ctx->tile_bits;
    const uint64_t chunk = uint64_t(1) << 28;  // blocks (bytes) per chunk, a multiple of 32
    const uint64_t nchunk = (nbytes + chunk - 1) / chunk;
    const uint64_t wpc = align_up(run_wpc(chunk), tb / 32);
    const DescLayout lay(1, 1);
    std::vector<uint8_t> host(lay.bytes * nchunk, 0);
    uint32_t *tmp = nullptr, *xf = nullptr;
    uint8_t *ddev = nullptr;
    CK(cudaMalloc(&tmp, size_t(8) * wpc * 4 + kMapPadBytes));
    CK(cudaMalloc(&xf, std::max<size_t>(size_t(8) * ctx->n_mid * 4, 4)));
    CK(cudaMalloc(&ddev, host.size()));
    const auto &pr = ctx->primes;
    std::vector<gbk::BatchParams> runs(nchunk);
    for (uint64_t c = 0; c < nchunk; ++c) {
        DescImage img;
        img.bind(host.data() + c * lay.bytes, lay);
        gbk::BatchParams &bb = img.runs[0];
        const uint64_t off = c * chunk;
        bb.base = lo + 30 * off;
        bb.nblk = uint32_t(std::min(chunk, nbytes - off));
        bb.qmax = bb.base + 30ull * bb.nblk;
        bb.wpc = uint32_t(wpc);
        bb.tiles_pc = uint32_t(wpc * 32 / tb);
        bb.tb_tiles = bb.tiles_pc;
        bb.tile_log2 = ctx->cfg.tile_log2;
        bb.tile_bits = tb;
        bb.tile_rcp = uint32_t(((uint64_t(1) << 32) + tb - 1) / tb);
        bb.map = tmp;
        bb.primes = ctx->d_primes;
        bb.magic = ctx->d_magic;
        bb.xfirst = xf;
        bb.pat = ctx->d_pat;
        bb.wheel = ctx->d_wheel;
        bb.pk_gap = ctx->d_pk_gap;
        bb.pk_base = ctx->d_pk_base;
        bb.pk_i0 = ctx->n_mid;
        bb.err = ctx->slot[0].err;
        bb.spin0 = gbk::kStageSpin;
        const uint64_t root = isqrt64(bb.qmax);
        bb.n_all = uint32_t(std::upper_bound(pr.begin(), pr.end(), root) - pr.begin());
        bb.i0 = std::min(ctx->i0, bb.n_all);
        bb.n_mid = std::max(std::min(ctx->n_mid, bb.n_all), bb.i0);
        bb.i_warp = std::min(std::max(ctx->i_warp, bb.i0), bb.n_mid);
        bb.n_hl = bb.n_all;
        set_residues(bb);
        img.h->nrun = 1;
        img.h->nseg = 0;
        finish_desc(ctx, img);
        runs[c] = bb;
    }
    cudaStream_t st = ctx->slot[0].st;
    CK(cudaMemcpy(ddev, host.data(), host.size(), cudaMemcpyHostToDevice));
    for (uint64_t c = 0; c < nchunk; ++c) {
        const gbk::BatchDesc d = lay.device(ddev + c * lay.bytes);
        gbh::launch_xfirst(d, ctx->grids, st);
        gbh::launch_tile(d, ctx->gi, ctx->tile_bits, ctx->tile_stage, ctx->grids, st);
        gbh::launch_large(d, ctx->grids, st);
        gbh::launch_wheel_bytes(runs[c], ctx->mtab + c * chunk / 4, st);
        ctx->launches += 4;
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    cudaFree(tmp);
    cudaFree(xf);
    cudaFree(ddev);
    ctx->mtab_m0 = lo;
    ctx->mtab_m1 = hi;
    ctx->mtab_builds += 1;
    ctx->mtab_build_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GBC_OK;
}

// multipliers [need0, need1] the hit-listed primes of a set of runs need
// (need0 > need1: none)
static void mtab_need(const gbc_ctx *ctx, const gbk::BatchParams *runs, uint32_t nrun, uint64_t &need0,
                      uint64_t &need1)
{
    need0 = UINT64_MAX;
    need1 = 0;
    for (uint32_t r = 0; r < nrun; ++r) {
        const gbk::BatchParams &bp = runs[r];
        if (bp.n_hl >= bp.n_all) continue;
        const uint64_t q1 = bp.base + 30ull * bp.nblk - 1;
        need0 = std::min(need0, bp.base / ctx->primes[bp.n_all - 1]);
        need1 = std::max(need1, q1 / ctx->primes[bp.n_hl]);
    }
}

extern "C" int gbc_prepare(gbc_ctx *ctx, uint64_t lo, uint64_t hi)
{
    if (!ctx || lo > hi || hi > ctx->cfg.limit) return fail(ctx, GBC_E_ARG, "need lo <= hi <= limit");
    if (!ctx->hl_on) return GBC_OK;
    // a run inside [lo, hi] has q in [base(lo), hi + 3 + 29] and sieving
    // primes up to sqrt(hi + 3): its hit-listed primes (from p_hl on) need
    // multipliers in [base(lo) / p_max, (hi + 32) / p_hl]
    const auto &pr = ctx->primes;
    const uint64_t qmax = hi + 3;
    const uint32_t n_all = uint32_t(std::upper_bound(pr.begin(), pr.end(), isqrt64(qmax)) - pr.begin());
    if (ctx->n_hl >= n_all) return GBC_OK;  // no hit-listed prime reaches hi
    const uint64_t s0 = std::max<uint64_t>(lo, 4);
    const uint64_t base = (s0 > GBC_MAX_CAND + 30 ? s0 - GBC_MAX_CAND : 0) / 30 * 30;
    return ensure_mtab(ctx, base / pr[n_all - 1], (qmax + 29) / pr[ctx->n_hl]);
}

// The plain form (launch mode 3): the batch's hit lists harvested and sorted
// once, as the reference harvests them once per batch of segments
// (src/verifier.cpp:1136-1143), then every segment in turn through the
// sieve, the large primes, the checkers and the count kernel, each launch
// narrowed to the segment by its header (plain_windows).
static int issue_plain(gbc_ctx *ctx, Slot &s)
{
    cudaStream_t st = s.st;
    const gbk::BatchDesc &d = s.dd;
    const gbh::Grids &g = ctx->grids;
    CK(cudaMemcpyAsync(s.desc_dev, s.desc_host, ctx->layout.bytes, cudaMemcpyHostToDevice, st));
    gbh::launch_init(d, g, st);
    gbh::launch_xfirst(d, g, st);
    gbh::launch_hitlist(d, false, g, st);
    gbh::launch_binsort(d, g, st);
    CK(cudaEventRecord(s.ev[1], st));
    const uint32_t nseg = s.img.h->nseg;
    for (uint32_t i = 0; i < nseg; ++i) {
        // the header sits at the descriptor's start
        CK(cudaMemcpyAsync(s.desc_dev, s.win_host + i, sizeof(gbk::BatchHeader), cudaMemcpyHostToDevice, st));
        gbh::launch_tile(d, ctx->gi, ctx->tile_bits, ctx->tile_stage, g, st);
        gbh::launch_large(d, g, st);
        gbh::launch_hitlist(d, true, g, st);
        gbh::launch_hl_overflow(d, g, st);
        gbh::launch_check(d, ctx->ct, g, st);
        gbh::launch_verify(d, ctx->vt, g, st);
        gbh::launch_retry(d, ctx->cfg.ridge_min, (ctx->cfg.test_flags & GBC_TEST_RETRY_LIMIT) ? 1u : (1u << 22), g,
                          st);
        gbh::launch_count(d, g, st);
    }
    // the stages interleave segment by segment: the sieve event takes the loop
    CK(cudaEventRecord(s.ev[2], st));
    CK(cudaEventRecord(s.ev[3], st));
    CK(cudaEventRecord(s.ev[4], st));
    ctx->launches += 4 + 9 * uint64_t(nseg);
    return GBC_OK;
}

// The pipeline of one batch on the slot's stream (the same calls are
// captured into the slot's graph): descriptor upload, result init, first
// bits, tiles | large primes, hit lists (filed by region, then applied
// region by region) | checker | counts.
static int issue_pipeline(gbc_ctx *ctx, Slot &s, bool capture)
{
    cudaStream_t st = s.st;
    const unsigned rec = capture ? cudaEventRecordExternal : cudaEventRecordDefault;
    const gbk::BatchDesc &d = s.dd;
    const gbh::Grids &g = ctx->grids;
    CK(cudaMemcpyAsync(s.desc_dev, s.desc_host, ctx->layout.bytes, cudaMemcpyHostToDevice, st));
    gbh::launch_init(d, g, st);
    gbh::launch_xfirst(d, g, st);
    gbh::launch_hitlist(d, false, g, st);  // binned batches: harvest into region bins
    gbh::launch_binsort(d, g, st);         // ... then into tile bins
    CK(cudaEventRecordWithFlags(s.ev[1], st, rec));
    gbh::launch_tile(d, ctx->gi, ctx->tile_bits, ctx->tile_stage, g, st);  // with the tile bins' marks
    gbh::launch_large(d, g, st);
    gbh::launch_hitlist(d, true, g, st);   // other batches: direct marks
    gbh::launch_hl_overflow(d, g, st);
    CK(cudaEventRecordWithFlags(s.ev[2], st, rec));
    gbh::launch_check(d, ctx->ct, g, st);
    gbh::launch_verify(d, ctx->vt, g, st);
    gbh::launch_retry(d, ctx->cfg.ridge_min, (ctx->cfg.test_flags & GBC_TEST_RETRY_LIMIT) ? 1u : (1u << 22), g, st);
    CK(cudaEventRecordWithFlags(s.ev[3], st, rec));
    gbh::launch_count(d, g, st);
    CK(cudaEventRecordWithFlags(s.ev[4], st, rec));
    return GBC_OK;
}

constexpr int kPipelineKernels = 14;

static int capture_slot(gbc_ctx *ctx, Slot &s)
{
    CK(cudaStreamBeginCapture(s.st, cudaStreamCaptureModeThreadLocal));
    const int r = issue_pipeline(ctx, s, true);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s.st, &graph);
    if (r) {
        if (graph) cudaGraphDestroy(graph);
        return r;
    }
    if (e != cudaSuccess) return fail(ctx, GBC_E_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    const cudaError_t e2 = cudaGraphInstantiate(&s.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e2 != cudaSuccess) {
        s.exec = nullptr;
        return fail(ctx, GBC_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e2));
    }
    return GBC_OK;
}

// Map self-check (the reference's enqueue_bucket_verify + map_compare,
// src/verifier.cpp:2057-2112): the batch's maps sieved again without hit
// lists (every prime above p_mid by the read-before-mark kernel) into a
// scratch buffer, then compared word by word; a mismatch sets an error flag.
static int issue_selfcheck(gbc_ctx *ctx, Slot &s)
{
    if (!s.chk_map) {
        CK(dev_alloc(ctx, &s.chk_map, s.map_words * 4 + kMapPadBytes));
        CK(cudaMemset(s.chk_map, 0, s.map_words * 4 + kMapPadBytes));
        CK(cudaMallocHost(&s.chk_desc_host, ctx->layout.bytes));
        CK(dev_alloc(ctx, &s.chk_desc_dev, ctx->layout.bytes));
        CK(dev_alloc(ctx, &s.chk_count, 4));
        s.chk_img.bind(s.chk_desc_host, ctx->layout);
        s.chk_dd = ctx->layout.device(s.chk_desc_dev);
    }
    std::memcpy(s.chk_desc_host, s.desc_host, ctx->layout.bytes);
    DescImage &ci = s.chk_img;
    for (uint32_t r = 0; r < ci.h->nrun; ++r) {
        gbk::BatchParams &bp = ci.runs[r];
        bp.map = s.chk_map + (bp.map - s.map);
        bp.n_hl = bp.n_all;
        bp.hl_quota = 0;
        bp.tb_cap = 0;
    }
    ci.h->n_hl_max = ci.h->n_all_max;
    ci.h->n_hl_min = ci.h->n_all_max;
    ci.h->nseg = 0;  // no checker work
    cudaStream_t st = s.st;
    CK(cudaMemcpyAsync(s.chk_desc_dev, s.chk_desc_host, ctx->layout.bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(s.chk_count, 0, 4, st));
    gbh::launch_tile(s.chk_dd, ctx->gi, ctx->tile_bits, ctx->tile_stage, ctx->grids, st);
    gbh::launch_large(s.chk_dd, ctx->grids, st);
    gbh::launch_map_compare(s.dd, s.chk_dd, s.chk_count, ctx->grids, st);
    ctx->launches += 3;
    ctx->selfchecks += 1;
    return GBC_OK;
}

static int enqueue_planned(gbc_ctx *ctx, Slot &s)
{
    const DescImage &img = s.img;
    uint64_t need0, need1;
    mtab_need(ctx, img.runs, img.h->nrun, need0, need1);
    const bool hl = need0 <= need1;
    if (hl) {
        if (int r = ensure_mtab(ctx, need0, need1)) return r;
        for (uint32_t r = 0; r < img.h->nrun; ++r) {
            img.runs[r].mtab = ctx->mtab;
            img.runs[r].m0 = ctx->mtab_m0;
            img.runs[r].m1 = ctx->mtab_m1;
        }
    }
    cudaStream_t st = s.st;
    CK(cudaEventRecord(s.ev[0], st));
    if (ctx->cfg.launch_mode == 3 && img.h->nrun == 1) {
        plain_windows(ctx, s);
        if (int r = issue_plain(ctx, s)) return r;
        ctx->launches -= kPipelineKernels;  // counted by issue_plain
    } else if (ctx->cfg.launch_mode >= 2) {
        if (int r = issue_pipeline(ctx, s, false)) return r;
    } else {
        if (!s.exec)
            if (int r = capture_slot(ctx, s)) return r;
        CK(cudaGraphLaunch(s.exec, st));
        ctx->graph_replays += 1;
    }
    ctx->launches += kPipelineKernels;
    s.did_selfcheck = false;
    if (hl) {
        ctx->hl_batches += 1;
        const uint32_t every = ctx->cfg.selfcheck_every;
        if (every && ctx->hl_batches % every == 0) {
            if (int r = issue_selfcheck(ctx, s)) return r;
            s.did_selfcheck = true;
        }
    }
    CK(cudaEventRecord(s.ev[5], st));
    CK(cudaGetLastError());
    s.nseg = int(img.h->nseg);
    s.nrun = int(img.h->nrun);
    s.pending = true;
    ctx->batches += 1;
    return GBC_OK;
}

extern "C" int gbc_enqueue_segments(gbc_ctx *ctx, int slot, const uint64_t *seg_bounds, const uint32_t *seg_flags,
                                    const uint64_t *seg_limits, int nseg)
{
    if (bad_slot(ctx, slot) || !seg_bounds || !seg_limits)
        return fail(ctx, GBC_E_ARG, "bad context, slot, bounds or limits");
    Slot &s = ctx->slot[slot];
    if (s.pending) return fail(ctx, GBC_E_STATE, "slot already holds an uncollected batch");
    if (int r = plan_batch(ctx, s, seg_bounds, seg_flags, seg_limits, nseg)) return r;
    return enqueue_planned(ctx, s);
}

extern "C" int gbc_enqueue_batch(gbc_ctx *ctx, int slot, const uint64_t *seg_bounds, const uint32_t *seg_flags,
                                 int nseg, uint64_t limit)
{
    if (bad_slot(ctx, slot) || !seg_bounds) return fail(ctx, GBC_E_ARG, "bad context, slot or bounds");
    if (nseg < 1 || uint32_t(nseg) > ctx->cfg.max_batch) return fail(ctx, GBC_E_ARG, "nseg outside [1, max_batch]");
    for (int i = 1; i < nseg; ++i)
        if (seg_bounds[2 * i] != seg_bounds[2 * i - 1] + 2) return fail(ctx, GBC_E_ARG, "segments must be consecutive");
    std::vector<uint64_t> lim(size_t(nseg), limit);
    return gbc_enqueue_segments(ctx, slot, seg_bounds, seg_flags, lim.data(), nseg);
}

extern "C" int gbc_poll(gbc_ctx *ctx, int slot)
{
    if (bad_slot(ctx, slot)) return fail(ctx, GBC_E_ARG, "bad context or slot");
    Slot &s = ctx->slot[slot];
    if (!s.pending) return 0;
    const cudaError_t q = cudaEventQuery(s.ev[5]);
    if (q == cudaSuccess) return 1;
    if (q == cudaErrorNotReady) return 0;
    return fail(ctx, GBC_E_CUDA, std::string("batch: ") + cudaGetErrorString(q));
}

extern "C" int gbc_collect(gbc_ctx *ctx, int slot, gbc_segment_result *out, int nseg, gbc_batch_times *times,
                           int timeout_ms)
{
    if (bad_slot(ctx, slot) || !out) return fail(ctx, GBC_E_ARG, "bad context, slot or output");
    Slot &s = ctx->slot[slot];
    if (!s.pending) return fail(ctx, GBC_E_STATE, "collect without an enqueued batch");
    if (nseg != s.nseg) return fail(ctx, GBC_E_ARG, "nseg differs from the enqueued batch");
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t q = cudaEventQuery(s.ev[5]);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) return fail(ctx, GBC_E_CUDA, std::string("batch: ") + cudaGetErrorString(q));
        if (timeout_ms >= 0 &&
            std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
            return fail(ctx, GBC_E_TIMEOUT, "batch not finished within the timeout");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    CK(cudaMemcpy(out, s.res, size_t(nseg) * sizeof(gbc_segment_result), cudaMemcpyDeviceToHost));
    uint32_t berr = 0, bad_words = 0;
    CK(cudaMemcpy(&berr, s.err, 4, cudaMemcpyDeviceToHost));
    if (s.did_selfcheck) CK(cudaMemcpy(&bad_words, s.chk_count, 4, cudaMemcpyDeviceToHost));
    if (ctx->cfg.hl_cap_pct < 100 && s.img.h->nrun && gbk::hl_binned(s.img.runs[0])) {
        uint32_t ov = 0;
        CK(cudaMemcpy(&ov, s.ovf_cnt, 4, cudaMemcpyDeviceToHost));
        ctx->hl_overflow += ov;
    }
    s.pending = false;
    if (berr) {
        char m[128];
        if (berr & gbk::kErrSelfCheck)
            std::snprintf(m, sizeof m, "map self-check: %u class-map words differ from the rebuild without hit lists",
                          bad_words);
        else std::snprintf(m, sizeof m, "device error flags 0x%x in the batch's sieve", berr);
        return fail(ctx, GBC_E_DEVICE, m);
    }
    if (times) {
        float a = 0, b = 0, c = 0, d = 0, e = 0;
        cudaEventElapsedTime(&a, s.ev[0], s.ev[1]);
        cudaEventElapsedTime(&b, s.ev[1], s.ev[2]);
        cudaEventElapsedTime(&c, s.ev[2], s.ev[3]);
        cudaEventElapsedTime(&d, s.ev[3], s.ev[4]);
        if (s.did_selfcheck) cudaEventElapsedTime(&e, s.ev[4], s.ev[5]);
        times->ms_setup = 0;
        times->ms_large = a;  // hit lists: harvest and sort
        times->ms_tile = b;   // the map: tiles with the sorted marks, large primes, other marks
        times->ms_check = c;
        times->ms_count = d;
        times->ms_selfcheck = e;
        times->ms_total = a + b + c + d + e;
        times->runs = uint32_t(s.nrun);
    }
    for (int i = 0; i < nseg; ++i) {
        gbc_segment_result &r = out[i];
        const gbk::SegParams &sp = s.img.segs[i];
        r.seg_start = sp.seg_start;
        r.seg_end = sp.seg_end;
        r.evens = (sp.seg_end - sp.seg_start) / 2 + 1;
        r.cnt_lo = sp.cnt_lo;
        r.cnt_hi = sp.cnt_hi;
        r.twin_hi = sp.twin_hi;
        r.hash_lo = sp.hash_lo;
        r.hash_hi = sp.hash_hi;
        r.sampled = sp.sampled;
        if (r.err) {
            char m[160];
            std::snprintf(m, sizeof m, "device error flags 0x%x in segment [%llu, %llu]", r.err,
                          (unsigned long long)sp.seg_start, (unsigned long long)sp.seg_end);
            return fail(ctx, GBC_E_DEVICE, m);
        }
        if (r.nleft > GBC_LEFT_CAP || r.ntail > GBC_TAIL_CAP || r.nridge > GBC_RIDGE_CAP || r.npend > s.pend_cap)
            return fail(ctx, GBC_E_OVERFLOW, "leftover, gap-tail, ridge or pending list overflow");
    }
    return GBC_OK;
}

extern "C" int gbc_copy_pn(gbc_ctx *ctx, int slot, int seg, uint16_t *out, uint64_t evens)
{
    if (bad_slot(ctx, slot) || !out) return fail(ctx, GBC_E_ARG, "bad arguments");
    Slot &s = ctx->slot[slot];
    if (!s.pn) return fail(ctx, GBC_E_STATE, "context made without want_pn");
    if (seg < 0 || seg >= s.nseg) return fail(ctx, GBC_E_ARG, "segment index");
    const gbk::SegParams &sp = s.img.segs[seg];
    if (evens != (sp.seg_end - sp.seg_start) / 2 + 1) return fail(ctx, GBC_E_ARG, "evens differs from the segment");
    CK(cudaMemcpyAsync(out, s.pn + size_t(seg) * s.pn_stride, evens * 2, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    return GBC_OK;
}

extern "C" int gbc_map_run(gbc_ctx *ctx, int slot, int run, uint64_t *base, uint32_t *nblk, uint32_t *wpc,
                           uint32_t *out, uint64_t out_words)
{
    if (bad_slot(ctx, slot)) return fail(ctx, GBC_E_ARG, "bad context or slot");
    Slot &s = ctx->slot[slot];
    if (s.pending) return fail(ctx, GBC_E_STATE, "the slot's batch is not collected yet");
    if (!s.nseg) return fail(ctx, GBC_E_STATE, "no batch on this slot yet");
    if (run < 0 || run >= s.nrun) return fail(ctx, GBC_E_ARG, "run index");
    const gbk::BatchParams &bp = s.img.runs[run];
    if (base) *base = bp.base;
    if (nblk) *nblk = bp.nblk;
    if (wpc) *wpc = bp.wpc;
    if (out) {
        if (out_words < uint64_t(8) * bp.wpc) return fail(ctx, GBC_E_ARG, "output smaller than 8 * wpc words");
        CK(cudaMemcpy(out, bp.map, size_t(8) * bp.wpc * 4, cudaMemcpyDeviceToHost));
    }
    return GBC_OK;
}

extern "C" int gbc_map_info(gbc_ctx *ctx, int slot, uint64_t *base, uint32_t *nblk, uint32_t *wpc, uint32_t *out,
                            uint64_t out_words)
{
    return gbc_map_run(ctx, slot, 0, base, nblk, wpc, out, out_words);
}

extern "C" const uint16_t *gbc_pn_device_ptr(gbc_ctx *ctx, int slot, int seg)
{
    if (bad_slot(ctx, slot)) return nullptr;
    Slot &s = ctx->slot[slot];
    if (!s.pn || seg < 0 || uint32_t(seg) >= ctx->cfg.max_batch) return nullptr;
    return s.pn + size_t(seg) * s.pn_stride;
}
