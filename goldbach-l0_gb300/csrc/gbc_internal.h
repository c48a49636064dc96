// gbc_internal.h -- the context and slot behind the opaque gbc_ctx of
// include/gbc.h (host side of the CUDA translation units only).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbc_common.cuh"

// Slack after the last class array: the checker stages up to 160 words past
// a class array's last used word, the count kernel reads 33.
constexpr size_t kMapPadBytes = 64 * 1024;

// Byte offsets of the parts of a batch descriptor for nrun_cap runs and
// nseg_cap segments (host image and device copy share the layout).
struct DescLayout {
    size_t runs = 0, segs = 0, tile_pref = 0, chk_pref = 0, ver_pref = 0, cnt_pref = 0, bytes = 0;
    DescLayout() = default;
    DescLayout(uint32_t nrun_cap, uint32_t nseg_cap);
    gbk::BatchDesc device(const uint8_t *base) const;
};

// Host-side view of a descriptor image.
struct DescImage {
    gbk::BatchHeader *h = nullptr;
    gbk::BatchParams *runs = nullptr;
    gbk::SegParams *segs = nullptr;
    uint32_t *tile_pref = nullptr, *chk_pref = nullptr, *ver_pref = nullptr, *cnt_pref = nullptr;
    void bind(uint8_t *base, const DescLayout &l);
};

// One independent set of device buffers with its own stream (the
// reference's pipeline slot, src/verifier.cpp:48-50).
struct Slot {
    cudaStream_t st = nullptr;
    // 0 start, 1 hit lists harvested and sorted, 2 map done (tiles, large
    // primes, direct and overflow marks), 3 checker done, 4 counts done (end
    // of the pipeline), 5 end of the batch (after a self-check)
    cudaEvent_t ev[6] = {};
    uint32_t *map = nullptr;           // class maps of the batch's runs, back to back
    size_t map_words = 0;              // capacity (words, without the pad)
    uint32_t *xfirst = nullptr;        // first class bits of the runs, back to back
    size_t xfirst_words = 0;
    gbc_segment_result *res = nullptr; // max_batch results
    uint32_t *err = nullptr;
    uint16_t *pn = nullptr;            // max_batch * pn_stride p(n), or nullptr
    uint64_t pn_stride = 0;
    uint2 *pend = nullptr;             // max_batch * pend_cap phase-A pending words
    uint32_t pend_cap = 0;
    // binned hit lists of one-run batches (k_hitlist's CTAs x region bins x quota)
    uint32_t *hl_buf = nullptr;
    size_t hl_buf_words = 0;
    uint32_t *hl_cnt = nullptr;
    // their tile bins (8 x tiles per class of a full run, tb_cap offsets
    // each) and the overflow list
    uint32_t *tb_buf = nullptr;
    size_t tb_buf_words = 0;
    uint32_t *tb_cnt = nullptr;
    size_t tb_cnt_words = 0;
    uint2 *ovf_buf = nullptr;
    uint32_t *ovf_cnt = nullptr;
    uint32_t ovf_cap = 0;
    // the batch descriptor: pinned host image, device copy
    uint8_t *desc_host = nullptr, *desc_dev = nullptr;
    // the plain form (launch mode 3): one header per segment of the batch,
    // each the batch's header narrowed to the segment (pinned, max_batch)
    gbk::BatchHeader *win_host = nullptr;
    DescImage img;
    gbk::BatchDesc dd{};
    cudaGraphExec_t exec = nullptr;    // the captured pipeline (launch modes 0 and 1)
    // map self-check: maps rebuilt without hit lists, their descriptor, mismatch count
    uint32_t *chk_map = nullptr;
    uint8_t *chk_desc_host = nullptr, *chk_desc_dev = nullptr;
    DescImage chk_img;
    gbk::BatchDesc chk_dd{};
    uint32_t *chk_count = nullptr;
    bool did_selfcheck = false;
    int nseg = 0, nrun = 0;
    bool pending = false;
};

struct gbc_ctx {
    gbc_config cfg{};
    gbh::Grids grids{};
    std::vector<uint32_t> primes;      // odd sieving primes ascending
    uint32_t i0 = 0, n_mid = 0, i_warp = 0;
    uint32_t wpc_cap = 0;              // class-array words of max_batch full segments in one run
    DescLayout layout;
    uint32_t *d_primes = nullptr, *d_magic = nullptr, *d_pat = nullptr;
    uint16_t *d_wheel = nullptr, *d_cand = nullptr, *d_list = nullptr;
    uint8_t *d_pk_gap = nullptr;   // packed large primes from n_mid: half gaps
    uint32_t *d_pk_base = nullptr; // and the first prime of each group
    uint2 *d_fun = nullptr, *d_fpair = nullptr;
    uint16_t *d_rest = nullptr;
    gbk::GroupInfo gi{};
    gbk::CheckTables ct{};
    gbk::VerifyTables vt{};
    std::vector<Slot> slot;
    std::string err;
    // host outputs of runs on this context (gb_records.cpp), owned
    void *outputs = nullptr;
    void (*outputs_del)(void *) = nullptr;
    // campaign statistics files of runs on this context (gb_stats.cpp), owned
    void *stats = nullptr;
    void (*stats_del)(void *) = nullptr;
    bool stats_gaps = true;
    uint64_t launches = 0, batches = 0, graph_replays = 0, selfchecks = 0, hl_batches = 0;
    uint32_t hl_overflow = 0;  // overflow-list marks seen by collect (hl_cap_pct < 100 only)
    uint64_t device_bytes = 0;
    // prime-multiplier table (hit lists for the primes >= p_hl)
    bool hl_on = false;
    uint64_t p_hl = 0;
    uint32_t tile_bits = 0;   // bits per tile of the persistent tile kernel
    uint32_t tile_stage = 0;  // tile-bin offsets it stages into shared memory
    uint32_t n_hl = 0;                 // index of the first prime >= p_hl
    uint32_t *mtab = nullptr;          // wheel-30 bytes of the primes in [mtab_m0, mtab_m1]
    uint64_t mtab_m0 = 0, mtab_m1 = 0, mtab_bytes = 0;
    uint64_t mtab_builds = 0;
    double mtab_build_ms = 0;
};

std::vector<uint32_t> gbh_odd_primes_upto(uint64_t n);
// the same, shared by the contexts of a process (the last list sieved is
// kept; a smaller bound takes a prefix of it)
std::vector<uint32_t> gbh_cached_primes(uint64_t n);
