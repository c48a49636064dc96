// gbc_internal.h -- the context and slot behind the opaque gbc_ctx of
// include/gbc.h (host side of the CUDA translation units only).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbc_common.cuh"

// Slack after the last class array: the checker's and the count kernel's
// warps read up to 33 words past a class array's last used word.
constexpr size_t kMapPadBytes = 64 * 1024;

// One of the two independent buffer sets (the reference's pipeline slot,
// src/verifier.cpp:48-50).
struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t ev[5] = {};
    uint32_t *map = nullptr;           // 8 * wpc_cap words + pad
    uint32_t *xfirst = nullptr;        // 8 * n_mid first class bits
    gbc_segment_result *res = nullptr; // max_batch results
    uint32_t *err = nullptr;
    uint16_t *pn = nullptr;            // max_batch * pn_stride p(n), or nullptr
    uint64_t pn_stride = 0;
    uint2 *pend = nullptr;             // max_batch * pend_cap phase-A pending words
    uint32_t pend_cap = 0;
    int nseg = 0;
    bool pending = false;
    gbk::BatchParams bp{};
    std::vector<gbk::SegParams> segs;
};

struct gbc_ctx {
    gbc_config cfg{};
    int sm_count = 1;
    std::vector<uint32_t> primes;      // odd sieving primes ascending
    uint32_t i0 = 0, n_mid = 0, i_warp = 0;
    uint32_t wpc_cap = 0;              // class-array words a slot holds
    uint32_t *d_primes = nullptr, *d_magic = nullptr, *d_pat = nullptr, *d_skip = nullptr;
    uint16_t *d_inv = nullptr, *d_cand = nullptr, *d_list = nullptr;
    uint32_t *d_fun = nullptr;
    uint16_t *d_rest = nullptr;
    gbk::GroupInfo gi{};
    gbk::CheckTables ct{};
    gbk::VerifyTables vt{};
    Slot slot[2];
    std::string err;
    uint64_t launches = 0;
    // prime-multiplier table (hit lists for the primes >= p_hl)
    bool hl_on = false;
    uint64_t p_hl = 0;
    uint32_t n_hl = 0;                 // index of the first prime >= p_hl
    uint32_t *mtab = nullptr;          // wheel-30 bytes of the primes in [mtab_m0, mtab_m1]
    uint64_t mtab_m0 = 0, mtab_m1 = 0;
    uint64_t mtab_builds = 0;
    double mtab_build_ms = 0;
};

std::vector<uint32_t> gbh_odd_primes_upto(uint64_t n);
int gbh_plan_batch(gbc_ctx *ctx, Slot &s, const uint64_t *bounds, const uint32_t *flags, int nseg, uint64_t limit,
                   gbk::BatchParams &bp);
