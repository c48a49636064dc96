// gb_sched.cpp -- the window scheduler (gb_sched.hpp), the batched
// uneven-window call gbc_verify_windows and the serving loop gbc_server_*
// of include/gbc.h.
#include "gb_sched.hpp"

#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <thread>

void gbh_set_error(gbc_ctx *ctx, const char *msg);  // gbc_api.cu

namespace gb {

namespace {

void check(gbc_ctx *ctx, int rc, const char *what)
{
    if (rc != GBC_OK) throw GbcError(rc, std::string(what) + ": " + gbc_last_error(ctx));
}

}  // namespace

Window::Window(uint64_t id_, uint64_t start_, uint64_t limit_, uint64_t segment_even, uint32_t sample_every)
    : id(id_), start(start_), limit(limit_), acc(start_, limit_)
{
    segs = plan_segments(start, limit, segment_even);
    flags.resize(segs.size());
    for (size_t j = 0; j < segs.size(); ++j) flags[j] = segment_flag(sample_every, j);
    t_submit = Clock::now();
}

RangeStats Window::stats() const
{
    RangeStats st;
    st.start = start;
    st.limit = limit;
    st.evens = acc.evens();
    st.segments = segs.size();
    st.batches = batches;
    st.leftovers = acc.leftovers();
    st.pmax = acc.pmax();
    st.primes = acc.primes();
    st.twins = acc.twins();
    st.evens_sampled = acc.evens_sampled();
    st.tail_evens = acc.tail_evens();
    st.pending = acc.pending();
    st.stats_line = acc.stats_ref_line();
    st.gbstats_line = acc.gbstats_line("gb300-1.0");
    st.ridges = acc.ridges();
    st.wall_seconds = std::chrono::duration<double>(t_done - t_submit).count();
    return st;
}

Scheduler::Scheduler(gbc_ctx *ctx) : ctx_(ctx)
{
    check(ctx, gbc_get_config(ctx, &cfg_), "config");
    for (int s = int(cfg_.nslots) - 1; s >= 0; --s) free_slots_.push_back(s);
    out_.resize(cfg_.max_batch);
}

void Scheduler::add(std::shared_ptr<Window> w)
{
    if (!w->segs.empty()) queue_.push_back(std::move(w));
}

int Scheduler::launch_ready()
{
    int launched = 0;
    while (!free_slots_.empty() && !queue_.empty()) {
        InFlight f;
        f.slot = free_slots_.back();
        std::vector<uint64_t> bounds, limits;
        std::vector<uint32_t> flags;
        uint32_t runs = 0;
        uint64_t prev_end = 0;
        bool have_prev = false;
        // windows in arrival order, each one's segments in order, until the
        // batch holds max_batch segments or max_runs runs
        while (!queue_.empty() && f.items.size() < cfg_.max_batch) {
            auto &w = queue_.front();
            const auto &s = w->segs[w->next];
            const bool joins = have_prev && s.first == prev_end + 2;
            if (!joins && runs == cfg_.max_runs) break;
            if (!joins) ++runs;
            bounds.push_back(s.first);
            bounds.push_back(s.second);
            limits.push_back(w->limit);
            flags.push_back(w->flags[w->next]);
            if (f.items.empty() || f.items.back().w != w) w->batches += 1;
            f.items.push_back({w, w->next});
            prev_end = s.second;
            have_prev = true;
            if (++w->next == w->segs.size()) queue_.pop_front();
        }
        check(ctx_, gbc_enqueue_segments(ctx_, f.slot, bounds.data(), flags.data(), limits.data(),
                                         int(f.items.size())),
              "enqueue");
        free_slots_.pop_back();
        st_.batches += 1;
        st_.segments += f.items.size();
        st_.runs += runs;
        inflight_.push_back(std::move(f));
        st_.max_in_flight = std::max(st_.max_in_flight, int(inflight_.size()));
        ++launched;
    }
    return launched;
}

std::vector<std::shared_ptr<Window>> Scheduler::finish(InFlight &f)
{
    const int n = int(f.items.size());
    gbc_batch_times tm{};
    check(ctx_, gbc_collect(ctx_, f.slot, out_.data(), n, &tm, 600000), "collect");
    st_.gpu_ms += tm.ms_total;
    free_slots_.push_back(f.slot);
    std::vector<std::shared_ptr<Window>> done;
    for (int i = 0; i < n; ++i) {
        auto &w = f.items[i].w;
        w->acc.add_segment(out_[i]);
        if (++w->done == w->segs.size()) {
            w->t_done = Clock::now();
            st_.windows += 1;
            done.push_back(w);
        }
    }
    return done;
}

std::vector<std::shared_ptr<Window>> Scheduler::collect(bool block)
{
    std::vector<std::shared_ptr<Window>> done;
    bool any = false;
    for (auto it = inflight_.begin(); it != inflight_.end();) {
        const int r = gbc_poll(ctx_, it->slot);
        if (r < 0) check(ctx_, r, "poll");
        if (r == 1) {
            auto d = finish(*it);
            done.insert(done.end(), d.begin(), d.end());
            it = inflight_.erase(it);
            any = true;
        } else ++it;
    }
    if (!any && block && !inflight_.empty()) {
        auto d = finish(inflight_.front());
        done.insert(done.end(), d.begin(), d.end());
        inflight_.pop_front();
    }
    return done;
}

std::vector<RangeStats> run_windows(gbc_ctx *ctx, const std::vector<std::pair<uint64_t, uint64_t>> &windows,
                                  SchedStats *out)
{
    gbc_config cfg{};
    check(ctx, gbc_get_config(ctx, &cfg), "config");
    Scheduler sch(ctx);
    std::vector<std::shared_ptr<Window>> ws;
    for (size_t i = 0; i < windows.size(); ++i) {
        uint64_t a = windows[i].first, b = windows[i].second;
        if (a < 4) a = 4;
        if (a & 1) a += 1;
        b &= ~uint64_t(1);
        if (b < 6 || a > b || b > cfg.limit)
            throw GbcError(GBC_E_ARG, "window " + std::to_string(i) + ": need 4 <= start <= limit <= context limit");
        ws.push_back(std::make_shared<Window>(i, a, b, cfg.segment_even, cfg.sample_every));
        sch.add(ws.back());
    }
    while (!sch.idle()) {
        sch.launch_ready();
        sch.collect(true);
    }
    std::vector<RangeStats> res;
    for (auto &w : ws) res.push_back(w->stats());
    if (out) *out = sch.stats();
    return res;
}

}  // namespace gb

namespace {

void fill_result(gbc_run_result *r, const gb::RangeStats &st)
{
    r->start = st.start;
    r->limit = st.limit;
    r->evens = st.evens;
    r->segments = st.segments;
    r->batches = st.batches;
    r->leftovers = st.leftovers;
    r->pmax = st.pmax;
    r->primes = st.primes;
    r->twins = st.twins;
    r->gpu_seconds = st.gpu_seconds;
    r->wall_seconds = st.wall_seconds;
}

// the stats_ref line when every segment was sampled, else the GBSTATS v2 line
int put_line(const gb::RangeStats &st, char *line, uint64_t cap)
{
    if (!line || !cap) return GBC_OK;
    const std::string &l = st.stats_line.empty() ? st.gbstats_line : st.stats_line;
    if (l.size() + 1 > cap) return GBC_E_OVERFLOW;
    std::memcpy(line, l.c_str(), l.size() + 1);
    return GBC_OK;
}

}  // namespace

extern "C" int gbc_verify_windows(gbc_ctx *ctx, const uint64_t *bounds, int nwin, gbc_run_result *res, char *lines,
                                  uint64_t line_stride, gbc_windows_summary *sum)
{
    if (!ctx || !bounds || nwin < 1) return GBC_E_ARG;
    try {
        std::vector<std::pair<uint64_t, uint64_t>> w;
        for (int i = 0; i < nwin; ++i) w.push_back({bounds[2 * i], bounds[2 * i + 1]});
        const auto t0 = gb::Clock::now();
        gb::SchedStats ss;
        const std::vector<gb::RangeStats> st = gb::run_windows(ctx, w, &ss);
        for (int i = 0; i < nwin; ++i) {
            if (res) fill_result(res + i, st[i]);
            if (lines)
                if (int rc = put_line(st[i], lines + uint64_t(i) * line_stride, line_stride)) return rc;
        }
        if (sum) {
            sum->batches = ss.batches;
            sum->segments = ss.segments;
            sum->runs = ss.runs;
            sum->gpu_seconds = ss.gpu_ms / 1e3;
            sum->wall_seconds = std::chrono::duration<double>(gb::Clock::now() - t0).count();
        }
        return GBC_OK;
    } catch (const gb::GbcError &e) {
        gbh_set_error(ctx, e.what());
        return e.code;
    } catch (const std::exception &e) {
        gbh_set_error(ctx, e.what());
        return GBC_E_DEVICE;
    }
}

// ---------------------------------------------------------------------------
// Serving loop: a worker thread owns the context and runs the scheduler;
// callers submit windows from any thread and wait for their results.
// ---------------------------------------------------------------------------
struct gbc_server {
    gbc_ctx *ctx = nullptr;
    gbc_config cfg{};
    uint64_t budget = 0;
    std::mutex mu;
    std::condition_variable cv_in, cv_done;
    std::deque<std::shared_ptr<gb::Window>> inbox;
    std::map<uint64_t, std::shared_ptr<gb::Window>> done;
    uint64_t next_id = 1, submitted = 0, completed = 0;
    bool stop = false;
    int error = GBC_OK;
    std::string error_msg;
    std::thread worker;
    gb::SchedStats stats;
    double busy_s = 0;
    gb::Clock::time_point t_start;
};

namespace {

void serve(gbc_server *srv)
{
    gb::Scheduler sch(srv->ctx);
    std::vector<std::shared_ptr<gb::Window>> fresh;
    try {
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(srv->mu);
                if (sch.idle() && srv->inbox.empty()) {
                    if (srv->stop) break;
                    srv->cv_in.wait_for(lk, std::chrono::milliseconds(50));
                }
                while (!srv->inbox.empty()) {
                    fresh.push_back(std::move(srv->inbox.front()));
                    srv->inbox.pop_front();
                }
            }
            for (auto &w : fresh) sch.add(std::move(w));
            fresh.clear();
            sch.launch_ready();
            auto fin = sch.collect(false);
            if (!fin.empty()) {
                std::lock_guard<std::mutex> lk(srv->mu);
                for (auto &w : fin) {
                    srv->done[w->id] = w;
                    srv->completed += 1;
                }
                srv->stats = sch.stats();
                srv->cv_done.notify_all();
            } else if (!sch.idle()) {
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            }
        }
    } catch (const gb::GbcError &e) {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->error = e.code;
        srv->error_msg = e.what();
    } catch (const std::exception &e) {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->error = GBC_E_DEVICE;
        srv->error_msg = e.what();
    }
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stats = sch.stats();
    srv->cv_done.notify_all();
}

}  // namespace

extern "C" int gbc_server_start(gbc_ctx *ctx, uint64_t hbm_budget, uint64_t lo, uint64_t hi, gbc_server **out)
{
    if (!ctx || !out) return GBC_E_ARG;
    *out = nullptr;
    gbc_config cfg{};
    if (gbc_get_config(ctx, &cfg) != GBC_OK) return GBC_E_ARG;
    // the table of prime multipliers for every window in [lo, hi], built now
    if (hi)
        if (int rc = gbc_prepare(ctx, lo, hi)) return rc;
    gbc_ctx_stats cs{};
    gbc_get_stats(ctx, &cs);
    if (hbm_budget && cs.device_bytes > hbm_budget) {
        gbh_set_error(ctx, "the context's device memory exceeds the HBM budget");
        return GBC_E_ARG;
    }
    auto *srv = new gbc_server();
    srv->ctx = ctx;
    srv->cfg = cfg;
    srv->budget = hbm_budget;
    srv->t_start = gb::Clock::now();
    srv->worker = std::thread(serve, srv);
    *out = srv;
    return GBC_OK;
}

extern "C" int gbc_server_submit(gbc_server *srv, uint64_t start, uint64_t limit, uint64_t *id)
{
    if (!srv) return GBC_E_ARG;
    if (start < 4) start = 4;
    if (start & 1) start += 1;
    limit &= ~uint64_t(1);
    if (limit < 6 || start > limit || limit > srv->cfg.limit) return GBC_E_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->error) return srv->error;
    if (srv->stop) return GBC_E_STATE;
    const uint64_t i = srv->next_id++;
    srv->inbox.push_back(
        std::make_shared<gb::Window>(i, start, limit, srv->cfg.segment_even, srv->cfg.sample_every));
    srv->submitted += 1;
    if (id) *id = i;
    srv->cv_in.notify_one();
    return GBC_OK;
}

extern "C" int gbc_server_wait(gbc_server *srv, uint64_t id, int timeout_ms, gbc_run_result *res, char *line,
                               uint64_t line_cap, double *latency_ms)
{
    if (!srv) return GBC_E_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    const auto deadline = gb::Clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
    for (;;) {
        auto it = srv->done.find(id);
        if (it != srv->done.end()) {
            auto w = it->second;
            srv->done.erase(it);
            lk.unlock();
            const gb::RangeStats st = w->stats();
            if (res) fill_result(res, st);
            if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(w->t_done - w->t_submit).count();
            return put_line(st, line, line_cap);
        }
        if (srv->error) return srv->error;
        if (timeout_ms < 0) srv->cv_done.wait(lk);
        else if (srv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !srv->done.count(id))
            return GBC_E_TIMEOUT;
    }
}

extern "C" int gbc_server_get_stats(gbc_server *srv, gbc_server_stats *out)
{
    if (!srv || !out) return GBC_E_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    out->submitted = srv->submitted;
    out->completed = srv->completed;
    out->batches = srv->stats.batches;
    out->segments = srv->stats.segments;
    out->runs = srv->stats.runs;
    out->max_in_flight = uint32_t(srv->stats.max_in_flight);
    out->gpu_seconds = srv->stats.gpu_ms / 1e3;
    out->wall_seconds = std::chrono::duration<double>(gb::Clock::now() - srv->t_start).count();
    gbc_ctx_stats cs{};
    gbc_get_stats(srv->ctx, &cs);
    out->device_bytes = cs.device_bytes;
    out->hbm_budget = srv->budget;
    return GBC_OK;
}

extern "C" const char *gbc_server_error(gbc_server *srv)
{
    if (!srv) return "no server";
    std::lock_guard<std::mutex> lk(srv->mu);
    return srv->error_msg.c_str();
}

extern "C" int gbc_server_stop(gbc_server *srv)
{
    if (!srv) return GBC_E_ARG;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
        srv->cv_in.notify_all();
    }
    if (srv->worker.joinable()) srv->worker.join();
    const int rc = srv->error;
    if (rc) gbh_set_error(srv->ctx, srv->error_msg.c_str());
    delete srv;
    return rc;
}
