// gb_sched.hpp -- continuous batching of verification windows over the
// slots of one gbc_ctx.
//
// The reference verifies one range at a time, one segment per slot
// (src/verifier.cpp:2487-2569). Here any number of windows of any width and
// height share the pipeline: their segments are queued in arrival order and
// packed into batches (up to max_batch segments in up to max_runs runs,
// one class map per run) on whichever slot is free, so a window that
// arrives while others are on the GPU starts in the next batch, and up to
// nslots batches overlap on the device, each on its own stream. Results are
// merged per window with the run driver's accumulator, so every window
// gets exactly the statistics a run of that window alone would give.
#pragma once
#include <chrono>
#include <cstdint>
#include <deque>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "gb_run.hpp"

namespace gb {

using Clock = std::chrono::steady_clock;

// One verification window and its merged results.
struct Window {
    uint64_t id = 0, start = 0, limit = 0;
    std::vector<std::pair<uint64_t, uint64_t>> segs;
    std::vector<uint32_t> flags;   // per segment: 0 (p(n) of every even) or GBC_SEG_VERIFY
    size_t next = 0;               // next segment to schedule
    size_t done = 0;               // segments collected
    uint64_t batches = 0;          // batches that held a segment of the window
    RunAccumulator acc;
    Clock::time_point t_submit, t_done;
    Window(uint64_t id, uint64_t start, uint64_t limit, uint64_t segment_even, uint32_t sample_every);
    bool finished() const { return done == segs.size(); }
    RangeStats stats() const;        // the window's RangeStats (lines, counts)
};

// Totals of a scheduler's life.
struct SchedStats {
    uint64_t batches = 0, segments = 0, runs = 0, windows = 0;
    double gpu_ms = 0;
    int max_in_flight = 0;
};

class Scheduler {
public:
    explicit Scheduler(gbc_ctx *ctx);
    void add(std::shared_ptr<Window> w);
    // nothing queued and nothing on the GPU
    bool idle() const { return queue_.empty() && inflight_.empty(); }
    bool has_queued() const { return !queue_.empty(); }
    // packs queued segments into batches on every free slot; returns how many
    int launch_ready();
    // collects every finished batch (block: wait for the oldest one if none
    // has finished); returns the windows that completed
    std::vector<std::shared_ptr<Window>> collect(bool block);
    const SchedStats &stats() const { return st_; }

private:
    struct Item {
        std::shared_ptr<Window> w;
        size_t seg;
    };
    struct InFlight {
        int slot;
        std::vector<Item> items;
    };
    std::vector<std::shared_ptr<Window>> finish(InFlight &f);

    gbc_ctx *ctx_;
    gbc_config cfg_{};
    std::deque<std::shared_ptr<Window>> queue_;  // windows with unscheduled segments
    std::deque<InFlight> inflight_;
    std::vector<int> free_slots_;
    std::vector<gbc_segment_result> out_;
    SchedStats st_;
};

// Verifies every window, segments packed across windows (the batched
// uneven-window form); returns each window's RangeStats in input order.
std::vector<RangeStats> run_windows(gbc_ctx *ctx, const std::vector<std::pair<uint64_t, uint64_t>> &windows,
                                  SchedStats *out = nullptr);

}  // namespace gb
