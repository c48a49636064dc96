// gb_records.cpp -- the run's host outputs besides its statistics line:
//   ridge store  the top 30 largest smallest-witness primes p(n) found so far,
//                one "rank,even,p,q,segment_start,found_unix" row each
//                (the reference's RidgeTracker store, include/ridge.hpp:
//                31-35, 196-237); every row entering it, from a run or from
//                the file, is proved on the CPU: p and n - p prime and no
//                smaller odd prime p' with n - p' prime
//   records      one line per notable event (include/gstats.hpp:836-868):
//                RECORD (p(n) above 9781, the largest p(n) known below
//                4e18), BEYOND (a p(n) outside the candidate list), SP (the
//                first even of the campaign whose p(n) is a prime whose first
//                occurrence S(p) is not known below 4e18); each re-proved by
//                an ascending Miller-Rabin scan, echoed to stderr, and handed
//                to a hook run in the background as `hook KIND P N Q CHECK`
//   live         a one-line JSON snapshot of the run in progress, rewritten
//                through a temporary file at most every 2 s
//                (include/gstats.hpp:775-820)
// The campaign's S(p) history is the records file itself: an SP line for p
// already there means S(p) was found before.
#include <algorithm>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "gb_run.hpp"

namespace gb {

namespace {

using u128 = unsigned __int128;

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return uint64_t(u128(a) * b % m); }

uint64_t powmod(uint64_t a, uint64_t e, uint64_t m)
{
    uint64_t r = 1;
    a %= m;
    while (e) {
        if (e & 1) r = mulmod(r, a, m);
        a = mulmod(a, a, m);
        e >>= 1;
    }
    return r;
}

// The primes p in 8423 .. 9769 whose first occurrence S(p) as a smallest
// Goldbach witness is not known below 4e18 (published search results; the
// reference's S_UNKNOWN_4E18, include/gstats.hpp:132-139), ascending.
const uint16_t kUnknownS[] = {
    8423, 8429, 8537, 8627, 8669, 8713, 8741, 8753, 8783, 8803, 8807, 8837, 8839, 8849, 8861, 8863, 8867, 8887,
    8893, 8923, 8963, 8969, 8999, 9007, 9011, 9013, 9029, 9041, 9043, 9049, 9059, 9067, 9103, 9109, 9127, 9133,
    9137, 9151, 9157, 9173, 9181, 9187, 9199, 9209, 9221, 9227, 9239, 9241, 9257, 9277, 9281, 9283, 9293, 9311,
    9319, 9323, 9337, 9343, 9349, 9371, 9377, 9391, 9397, 9403, 9413, 9419, 9421, 9431, 9433, 9437, 9439, 9461,
    9463, 9467, 9473, 9479, 9491, 9497, 9511, 9521, 9533, 9539, 9547, 9551, 9587, 9601, 9613, 9619, 9623, 9631,
    9643, 9649, 9661, 9677, 9679, 9689, 9697, 9719, 9721, 9733, 9739, 9743, 9749, 9767, 9769};
constexpr uint64_t kRecordP = 9781;  // the largest p(n) known below 4e18

bool write_atomically(const std::string &path, const std::string &text)
{
    const std::string tmp = path + ".tmp";
    std::FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
    if (std::fclose(f) != 0 || !ok) {
        std::remove(tmp.c_str());
        return false;
    }
    return std::rename(tmp.c_str(), path.c_str()) == 0;
}

}  // namespace

// Deterministic for every 64-bit n: the first twelve primes as bases suffice
// below 3.3e24 (Sorenson and Webster, 2015).
bool is_prime_u64(uint64_t n)
{
    if (n < 2) return false;
    static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (uint64_t p : small)
        if (n % p == 0) return n == p;
    uint64_t d = n - 1;
    int s = 0;
    while (!(d & 1)) {
        d >>= 1;
        ++s;
    }
    for (uint64_t a : small) {
        uint64_t x = powmod(a, d, n);
        if (x == 1 || x == n - 1) continue;
        bool comp = true;
        for (int r = 1; r < s && comp; ++r) {
            x = mulmod(x, x, n);
            if (x == n - 1) comp = false;
        }
        if (comp) return false;
    }
    return true;
}

uint64_t pn_exact(uint64_t n)
{
    if (n < 6 || (n & 1)) return 0;
    for (uint64_t p = 3; p <= n / 2; p += 2)
        if (is_prime_u64(p) && is_prime_u64(n - p)) return p;
    return 0;
}

// ---------------------------------------------------------------------------
// ridge store

static bool ridge_before(const RidgeRow &a, const RidgeRow &b) { return a.p != b.p ? a.p > b.p : a.n > b.n; }

bool RidgeStore::consider(uint64_t n, uint64_t p, uint64_t seg, uint64_t found)
{
    if (p < floor_) return false;
    ++appends_;
    if (n < 6 || (n & 1) || p < 3 || !(p & 1) || p >= n) {
        ++dropped_;
        return false;
    }
    if (top_.size() >= kKeep) {
        const RidgeRow &last = top_.back();
        if (p < last.p || (p == last.p && n <= last.n)) return false;
    }
    for (const RidgeRow &t : top_)
        if (t.n == n) return false;  // stored already: its first time stays
    if (!is_prime_u64(p) || !is_prime_u64(n - p)) {
        ++dropped_;
        return false;
    }
    for (uint64_t pp = 3; pp < p; pp += 2)  // minimality: no smaller witness
        if (is_prime_u64(pp) && is_prime_u64(n - pp)) {
            ++dropped_;
            return false;
        }
    if (found == UINT64_MAX) found = uint64_t(std::time(nullptr));
    const RidgeRow e{n, p, n - p, seg, found};
    top_.insert(std::upper_bound(top_.begin(), top_.end(), e, ridge_before), e);
    if (top_.size() > kKeep) top_.pop_back();
    changed_ = true;
    return true;
}

bool RidgeStore::load(const std::string &path)
{
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    char line[256];
    while (std::fgets(line, sizeof line, f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        unsigned long long r, n, p, q, s, t = 0;
        if (std::sscanf(line, "%llu,%llu,%llu,%llu,%llu,%llu", &r, &n, &p, &q, &s, &t) >= 5) consider(n, p, s, t);
    }
    std::fclose(f);
    changed_ = false;
    return true;
}

bool RidgeStore::save(const std::string &path)
{
    if (!changed_ || path.empty()) return true;
    std::string out =
        "# largest Goldbach ridges: the top 30 smallest-witness primes p of evens n = p + q\n"
        "# rank,even,small_prime_p,large_prime_q,segment_start,found_unix\n";
    char row[192];
    for (size_t i = 0; i < top_.size(); ++i) {
        const RidgeRow &e = top_[i];
        std::snprintf(row, sizeof row, "%zu,%" PRIu64 ",%" PRIu64 ",%" PRIu64 ",%" PRIu64 ",%" PRIu64 "\n", i + 1,
                      e.n, e.p, e.q, e.seg, e.found);
        out += row;
    }
    if (!write_atomically(path, out)) {
        std::fprintf(stderr, "ridge store: cannot write %s\n", path.c_str());
        return false;
    }
    changed_ = false;
    return true;
}

// ---------------------------------------------------------------------------
// records and the live snapshot

Outputs::Outputs(const char *ridge_csv, const char *records, const char *live_json, const char *hook,
                 uint32_t ridge_floor)
    : ridge_csv_(ridge_csv ? ridge_csv : ""), records_(records ? records : ""),
      live_json_(live_json ? live_json : ""), hook_(hook ? hook : ""), ridges_(ridge_floor)
{
    if (!ridge_csv_.empty()) ridges_.load(ridge_csv_);
    // S(p) found before: the records file's SP lines
    if (!records_.empty()) {
        std::ifstream in(records_);
        std::string line;
        while (std::getline(in, line)) {
            const size_t k = line.find(" p(n)=");
            if (k == std::string::npos || line.find("S(p) candidate") == std::string::npos) continue;
            sp_seen_.insert(std::strtoull(line.c_str() + k + 6, nullptr, 10));
        }
    }
}

void Outputs::record(uint64_t n, uint64_t p, const char *kind, const char *what)
{
    const uint64_t ex = pn_exact(n);
    const char *check = ex == p ? "OK" : "MISMATCH";
    const std::time_t t = std::time(nullptr);
    std::tm tm{};
    localtime_r(&t, &tm);
    char ts[32];
    std::strftime(ts, sizeof ts, "%Y-%m-%dT%H:%M:%S", &tm);
    char line[512];
    std::snprintf(line, sizeof line, "%s p(n)=%" PRIu64 " n=%" PRIu64 " q=%" PRIu64 " cpu_check=%s  %s\n", ts, p, n,
                  n - p, check, what);
    std::fprintf(stderr, "\n*** %s", line);
    if (!records_.empty())
        if (std::FILE *f = std::fopen(records_.c_str(), "ab")) {
            std::fputs(line, f);
            std::fclose(f);
        }
    events_.push_back({n, p});
    if (!hook_.empty()) {
        char cmd[1024];
        std::snprintf(cmd, sizeof cmd, "%s %s %" PRIu64 " %" PRIu64 " %" PRIu64 " %s >/dev/null 2>&1 &", hook_.c_str(),
                      kind, p, n, n - p, check);
        if (std::system(cmd) != 0) std::fprintf(stderr, "record hook failed to start: %s\n", hook_.c_str());
    }
}

void Outputs::note_beyond(uint64_t n, uint64_t p)
{
    if (p > kRecordP) record(n, p, "RECORD", "NEW RECORD: p(n) > 9781, the largest p(n) known below 4e18");
    else record(n, p, "BEYOND", "p(n) beyond the candidate list");
}

void Outputs::note_first(uint64_t n, uint64_t p)
{
    if (p > 0xFFFF || !std::binary_search(std::begin(kUnknownS), std::end(kUnknownS), uint16_t(p))) return;
    if (!sp_seen_.insert(p).second) return;
    record(n, p, "SP",
           "S(p) candidate: first even in this campaign with p(n) = p; S(p) was unknown (> 4e18) -- this IS S(p) "
           "if the campaign covers [4e18, n] without a gap");
}

void Outputs::add_segment(const gbc_segment_result &r, const std::vector<uint16_t> &cand)
{
    for (uint32_t i = 0; i < r.nridge && i < GBC_RIDGE_CAP; ++i) ridges_.consider(r.ridge_n[i], r.ridge_p[i], r.seg_start);
    for (uint32_t i = 0; i < r.nleft && i < GBC_LEFT_CAP; ++i) {
        const uint64_t p = r.left_p[i];
        ridges_.consider(r.left_n[i], p, r.seg_start);
        note_beyond(r.left_n[i], p);
    }
    for (size_t i = 0; i < cand.size() && i < size_t(GBC_NCAND); ++i)
        if (r.first[i] != 0xFFFFFFFFu) note_first(r.seg_start + 2ull * r.first[i], cand[i]);
}

void Outputs::write_live(uint64_t start, uint64_t limit, uint64_t evens_done, uint64_t evens_total, double elapsed,
                         const RunAccumulator &acc, bool force)
{
    if (live_json_.empty()) return;
    const std::time_t now = std::time(nullptr);
    if (!force && now - live_t_ < 2) return;
    live_t_ = now;
    const auto pm = acc.pmax_first();
    std::string o;
    char b[640];
    std::snprintf(b, sizeof b,
                  "{\"time\": %lld, \"start\": %" PRIu64 ", \"limit\": %" PRIu64 ", \"evens_done\": %" PRIu64
                  ", \"evens_total\": %" PRIu64 ", \"elapsed_s\": %.1f, \"tail_t\": %u, \"tail_evens\": %" PRIu64
                  ", \"pmax\": %" PRIu64 ", \"pmax_n\": %" PRIu64 ", \"ge8000\": %" PRIu64 ", \"ge9000\": %" PRIu64
                  ", \"gt9781\": %" PRIu64 ", \"primes\": %" PRIu64 ", \"twins\": %" PRIu64 ", \"events\": [",
                  (long long)now, start, limit, evens_done, evens_total, elapsed, GBC_TAIL_T, acc.tail_evens(),
                  pm.first, pm.second, acc.count_ge(8000), acc.count_ge(9000), acc.count_ge(kRecordP + 1),
                  acc.primes(), acc.twins());
    o += b;
    for (size_t i = 0; i < events_.size(); ++i) {
        std::snprintf(b, sizeof b, "%s[%" PRIu64 ", \"%" PRIu64 "\"]", i ? ", " : "", events_[i].second,
                      events_[i].first);
        o += b;
    }
    o += "]}\n";
    write_atomically(live_json_, o);
}

void Outputs::finish_run() { ridges_.save(ridge_csv_); }

}  // namespace gb

void *gbh_outputs(gbc_ctx *ctx);  // gbc_api.cu

gb::Outputs *gb::outputs_of(gbc_ctx *ctx) { return static_cast<gb::Outputs *>(gbh_outputs(ctx)); }

// The run's ridge store, records file and live snapshot at the reference's
// paths (src/verifier.cpp:725-745, include/gstats.hpp:474-478):
// GB_RIDGE_FILE (goldbach_ridges.csv; GB_RIDGE=0 turns ridges off),
// GB_RECORDS_FILE (goldbach_records.txt), GB_STATS_LIVE (goldbach_live.json);
// a variable set but empty turns its output off. The record hook is
// GB_RECORD_HOOK (set but empty: none), else scripts/notify_record.sh when
// present.
void gb::attach_env_outputs(gbc_ctx *ctx)
{
    auto path = [](const char *var, const char *def) -> std::string {
        const char *v = std::getenv(var);
        return v ? v : def;
    };
    const char *rg = std::getenv("GB_RIDGE");
    const bool ridge_on = !(rg && (!std::strcmp(rg, "0") || !std::strcmp(rg, "off")));
    const std::string ridge = ridge_on ? path("GB_RIDGE_FILE", "goldbach_ridges.csv") : "";
    const std::string rec = path("GB_RECORDS_FILE", "goldbach_records.txt");
    const std::string live = path("GB_STATS_LIVE", "goldbach_live.json");
    const char *hk = std::getenv("GB_RECORD_HOOK");
    std::string hook = hk ? hk : "";
    if (!hk)
        if (std::FILE *f = std::fopen("scripts/notify_record.sh", "rb")) {
            std::fclose(f);
            hook = "bash scripts/notify_record.sh";
        }
    if (gbc_set_outputs(ctx, ridge.c_str(), rec.c_str(), live.c_str(), hook.c_str()) != GBC_OK)
        std::fprintf(stderr, "outputs: %s\n", gbc_last_error(ctx));
}


// ---------------------------------------------------------------------------
// C ABI

void gbh_set_outputs(gbc_ctx *ctx, void *p, void (*del)(void *));  // gbc_api.cu
void gbh_set_error(gbc_ctx *ctx, const char *msg);                 // gbc_api.cu

extern "C" int gbc_set_outputs(gbc_ctx *ctx, const char *ridge_csv, const char *records, const char *live_json,
                               const char *hook)
{
    if (!ctx) return GBC_E_ARG;
    gbc_config cfg{};
    if (gbc_get_config(ctx, &cfg) != GBC_OK) return GBC_E_ARG;
    const bool any = (ridge_csv && *ridge_csv) || (records && *records) || (live_json && *live_json);
    if (!any) {
        gbh_set_outputs(ctx, nullptr, nullptr);
        return GBC_OK;
    }
    try {
        auto *o = new gb::Outputs(ridge_csv, records, live_json, hook, cfg.ridge_min);
        gbh_set_outputs(ctx, o, [](void *q) { delete static_cast<gb::Outputs *>(q); });
        return GBC_OK;
    } catch (const std::exception &e) {
        gbh_set_error(ctx, e.what());
        return GBC_E_ARG;
    }
}

extern "C" int gbc_ridges_merge(const char *path, const uint64_t *n, const uint64_t *p, const uint64_t *seg,
                                uint32_t count, uint32_t floor, uint32_t *kept)
{
    if (!path || !*path || (count && (!n || !p))) return GBC_E_ARG;
    gb::RidgeStore st(floor ? floor : 3);
    st.load(path);
    for (uint32_t i = 0; i < count; ++i) st.consider(n[i], p[i], seg ? seg[i] : 0);
    if (!st.save(path)) return GBC_E_ARG;
    if (kept) *kept = uint32_t(st.top().size());
    return GBC_OK;
}

extern "C" int gbc_record_event(const char *records, const char *hook, uint64_t n, uint64_t p, int first)
{
    if (!records || !*records) return GBC_E_ARG;
    gb::Outputs o(nullptr, records, nullptr, hook, 3);
    if (first) o.note_first(n, p);
    else o.note_beyond(n, p);
    return GBC_OK;
}

extern "C" uint64_t gbc_pn_exact(uint64_t n) { return gb::pn_exact(n); }
