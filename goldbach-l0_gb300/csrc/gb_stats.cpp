// gb_stats.cpp -- the campaign statistics files (gb_stats.hpp).
//
// The file formats, the merge rules and the refusal rules follow the
// reference's GoldbachStats (include/gstats.hpp): the strict record parsers
// of 319-395, GapStats::merge 436-451, commit 715-772, log_line and
// gap_fields 913-989, log_has_gaps_in 1000-1020, commit_gaps 1022-1064,
// load_gaps 1076-1153, load_state 1190-1272, save_state 1274-1313 and the
// durable replace 1315-1342. The code is this repository's own.
#include "gb_stats.hpp"

#include <fcntl.h>
#include <sys/file.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

#include "../../include/gbc.h"

namespace gb {

namespace {

constexpr int kClasses = GBC_NCLASS;
constexpr int kCand = GBC_NCAND;

const std::vector<uint16_t> &cands()
{
    static const std::vector<uint16_t> c = [] {
        std::vector<uint16_t> v(kCand);
        gbc_candidates(v.data(), kCand);
        return v;
    }();
    return c;
}

// candidate index of an odd p, or -1
int cand_index(uint64_t p)
{
    const auto &c = cands();
    const auto it = std::lower_bound(c.begin(), c.end(), p);
    return it != c.end() && *it == p ? int(it - c.begin()) : -1;
}

std::string u128_str(u128 v)
{
    std::string s;
    do {
        s.insert(s.begin(), char('0' + int(v % 10)));
        v /= 10;
    } while (v);
    return s;
}

// counts, comma-separated, an empty entry for 0, trailing zeros cut
std::string dense(const std::vector<uint64_t> &v, size_t from = 0)
{
    size_t last = 0;
    for (size_t i = from; i < v.size(); ++i)
        if (v[i]) last = i + 1;
    std::string s;
    for (size_t i = from; i < last; ++i) {
        if (i > from) s += ',';
        if (v[i]) s += std::to_string(v[i]);
    }
    return s;
}

// ---- strict parsing: plain decimal fields separated by single spaces ------

std::vector<std::string> fields(const std::string &line)
{
    std::vector<std::string> f;
    size_t pos = 0;
    for (;;) {
        const size_t e = line.find(' ', pos);
        f.push_back(line.substr(pos, e == std::string::npos ? std::string::npos : e - pos));
        if (e == std::string::npos) return f;
        pos = e + 1;
    }
}

bool parse_u128(const std::string &t, u128 &v)
{
    if (t.empty()) return false;
    const u128 max = ~u128(0);
    v = 0;
    for (char ch : t) {
        if (ch < '0' || ch > '9') return false;
        const unsigned d = unsigned(ch - '0');
        if (v > (max - d) / 10) return false;
        v = v * 10 + d;
    }
    return true;
}

bool parse_u64(const std::string &t, uint64_t &v)
{
    u128 w = 0;
    if (!parse_u128(t, w) || w > u128(UINT64_MAX)) return false;
    v = uint64_t(w);
    return true;
}

bool parse_u32(const std::string &t, uint32_t &v)
{
    uint64_t w = 0;
    if (!parse_u64(t, w) || w > UINT32_MAX) return false;
    v = uint32_t(w);
    return true;
}

// a dense list of at most n entries
bool parse_dense(const std::string &t, size_t n, std::vector<uint64_t> &v)
{
    v.assign(n, 0);
    if (t.empty()) return true;
    size_t i = 0, pos = 0;
    for (;;) {
        const size_t e = t.find(',', pos);
        const std::string x = t.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
        if (i >= n || (!x.empty() && !parse_u64(x, v[i]))) return false;
        ++i;
        if (e == std::string::npos) return true;
        pos = e + 1;
    }
}

void merge_ranges(std::vector<std::pair<uint64_t, uint64_t>> &r)
{
    std::sort(r.begin(), r.end());
    std::vector<std::pair<uint64_t, uint64_t>> m;
    for (const auto &c : r) {
        if (!m.empty() && c.first <= m.back().second + 2) m.back().second = std::max(m.back().second, c.second);
        else m.push_back(c);
    }
    r = m;
}

bool read_file(const std::string &path, std::string &all)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) return false;
    std::ostringstream ss;
    ss << in.rdbuf();
    all = ss.str();
    return true;
}

// temporary file, fsync, rename over path, fsync of the directory
void write_durably(const std::string &path, const std::string &out)
{
    const std::string tmp = path + ".tmp";
    std::FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) throw std::runtime_error("stats: cannot write " + tmp);
    bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    ok = std::fflush(f) == 0 && ok;
    ok = ::fsync(::fileno(f)) == 0 && ok;
    ok = std::fclose(f) == 0 && ok;
    if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        throw std::runtime_error("stats: cannot write " + path + " (state unchanged)");
    }
    const size_t sl = path.find_last_of('/');
    const std::string dir = sl == std::string::npos ? "." : (sl == 0 ? "/" : path.substr(0, sl));
    const int dfd = ::open(dir.c_str(), O_RDONLY | O_DIRECTORY | O_CLOEXEC);
    if (dfd >= 0) {
        ::fsync(dfd);
        ::close(dfd);
    }
}

// appended and flushed to disk; the state is authoritative, so a failed
// append only warns
void append_log(const std::string &path, const std::string &line)
{
    std::FILE *f = std::fopen(path.c_str(), "ab");
    if (!f) {
        std::fprintf(stderr, "stats: cannot append to %s\n", path.c_str());
        return;
    }
    bool ok = std::fwrite(line.data(), 1, line.size(), f) == line.size();
    ok = std::fflush(f) == 0 && ok;
    ok = ::fsync(::fileno(f)) == 0 && ok;
    if (std::fclose(f) != 0 || !ok) std::fprintf(stderr, "stats: incomplete append to %s\n", path.c_str());
}

struct FileLock {
    int fd = -1;
    explicit FileLock(const std::string &path)
    {
        fd = ::open(path.c_str(), O_RDWR | O_CREAT | O_CLOEXEC, 0644);
        if (fd < 0 || ::flock(fd, LOCK_EX) != 0) {
            if (fd >= 0) ::close(fd);
            throw std::runtime_error("stats: cannot lock " + path);
        }
    }
    ~FileLock() { ::close(fd); }
    FileLock(const FileLock &) = delete;
    FileLock &operator=(const FileLock &) = delete;
};

// ---- the campaign state -----------------------------------------------------

struct Campaign {
    std::vector<uint64_t> samp = std::vector<uint64_t>(size_t(kClasses) * kCand, 0);
    std::vector<uint64_t> tail_cls = std::vector<uint64_t>(size_t(kClasses) * kCand, 0);
    std::vector<uint64_t> tail_agg = std::vector<uint64_t>(kCand, 0);
    std::vector<uint64_t> first = std::vector<uint64_t>(kCand, 0);
    std::vector<std::pair<uint64_t, uint64_t>> covered;
    std::vector<std::pair<uint64_t, uint64_t>> beyond;  // (n, p)
    uint64_t evens = 0, sampled = 0, primes30[8] = {}, twins30[3] = {};
};

std::runtime_error damaged(const std::string &path, const std::string &line)
{
    return std::runtime_error("stats: state " + path + " has a malformed record '" + line.substr(0, 80) +
                              "' (damaged); refusing to merge into it");
}

Campaign load_state(const std::string &path, uint32_t tail_t)
{
    Campaign c;
    std::string all;
    if (!read_file(path, all)) return c;
    if (all.empty() || all.back() != '\n')
        throw std::runtime_error("stats: state " + path +
                                 " is empty or cut off (truncated write?); refusing to merge into it");
    uint32_t seen_samp = 0, seen_tail = 0;
    bool seen_t = false, seen_ev = false, seen_p = false, seen_tw = false, seen_agg = false;
    const auto once = [&](bool &seen, const std::string &ln) {
        if (seen) throw damaged(path, ln);
        seen = true;
    };
    size_t pos = 0;
    while (pos < all.size()) {
        const size_t e = all.find('\n', pos);
        const std::string ln = all.substr(pos, e - pos);
        pos = e + 1;
        if (ln.empty() || ln[0] == '#') continue;
        const std::vector<std::string> f = fields(ln);
        const std::string &k = f[0];
        const size_t nf = f.size();
        bool ok = true;
        uint64_t a = 0, b = 0;
        uint32_t p = 0, cr = 0;
        if (k == "range" && nf == 3) {
            ok = parse_u64(f[1], a) && parse_u64(f[2], b) && a <= b;
            c.covered.push_back({a, b});
        } else if (k == "tail_t" && nf == 2) {
            once(seen_t, ln);
            ok = parse_u32(f[1], p);
            if (ok && p != tail_t)
                throw std::runtime_error("stats: state " + path + " was recorded with tail_t " + std::to_string(p) +
                                         ", this run uses " + std::to_string(tail_t));
        } else if (k == "evens" && nf == 3) {
            once(seen_ev, ln);
            ok = parse_u64(f[1], c.evens) && parse_u64(f[2], c.sampled);
        } else if (k == "first" && nf == 3) {
            ok = parse_u32(f[1], p) && parse_u64(f[2], a);
            const int i = ok ? cand_index(p) : -1;
            ok = ok && i >= 0;
            if (ok) c.first[size_t(i)] = a;
        } else if (k == "beyond" && nf == 3) {
            ok = parse_u64(f[1], b) && parse_u64(f[2], a);
            c.beyond.push_back({a, b});
        } else if (k == "primes30" && nf == 9) {
            once(seen_p, ln);
            for (size_t i = 0; i < 8 && ok; ++i) ok = parse_u64(f[1 + i], c.primes30[i]);
        } else if (k == "twins30" && nf == 4) {
            once(seen_tw, ln);
            for (size_t i = 0; i < 3 && ok; ++i) ok = parse_u64(f[1 + i], c.twins30[i]);
        } else if ((k == "sampled" || k == "tailcls") && nf == 3) {
            uint32_t &seen = k == "sampled" ? seen_samp : seen_tail;
            std::vector<uint64_t> v;
            ok = parse_u32(f[1], cr) && cr < uint32_t(kClasses) && !((seen >> cr) & 1u) && parse_dense(f[2], kCand, v);
            if (ok) {
                std::copy(v.begin(), v.end(), (k == "sampled" ? c.samp : c.tail_cls).begin() + size_t(cr) * kCand);
                seen |= 1u << cr;
            }
        } else if (k == "tailagg" && nf == 2) {
            once(seen_agg, ln);
            ok = parse_dense(f[1], kCand, c.tail_agg);
        } else {
            ok = false;  // unknown record or wrong field count
        }
        if (!ok) throw damaged(path, ln);
    }
    if (!(seen_t && seen_ev && seen_p && seen_tw && seen_agg && seen_samp == 0x7FFFu && seen_tail == 0x7FFFu))
        throw std::runtime_error("stats: state " + path +
                                 " is missing records (truncated or damaged); refusing to merge into it");
    merge_ranges(c.covered);
    return c;
}

void save_state(const std::string &path, const Campaign &c, uint32_t tail_t)
{
    const auto &cand = cands();
    std::string o =
        "# goldbach-l0 statistics state v2 (exact; include/gstats.hpp)\n"
        "# lists: counts by odd-prime index (3, 5, 7, 11, ...), empty = 0\n"
        "# sampled <n mod 30 / 2>: p(n) histogram of the sampled segments\n"
        "# tailcls <n mod 30 / 2> / tailagg: p(n) >= tail_t, all evens (tailagg: class not kept)\n"
        "# first <p> <n>: first even of the campaign with p(n) = p (tail p only)\n";
    o += "tail_t " + std::to_string(tail_t) + "\n";
    for (const auto &r : c.covered) o += "range " + std::to_string(r.first) + " " + std::to_string(r.second) + "\n";
    o += "evens " + std::to_string(c.evens) + " " + std::to_string(c.sampled) + "\n";
    o += "primes30";
    for (uint64_t v : c.primes30) o += " " + std::to_string(v);
    o += "\ntwins30";
    for (uint64_t v : c.twins30) o += " " + std::to_string(v);
    o += "\n";
    for (int i = 0; i < kCand; ++i)
        if (c.first[size_t(i)]) o += "first " + std::to_string(cand[size_t(i)]) + " " + std::to_string(c.first[size_t(i)]) + "\n";
    for (const auto &b : c.beyond) o += "beyond " + std::to_string(b.second) + " " + std::to_string(b.first) + "\n";
    for (int cr = 0; cr < kClasses; ++cr)
        o += "sampled " + std::to_string(cr) + " " +
             dense(std::vector<uint64_t>(c.samp.begin() + size_t(cr) * kCand, c.samp.begin() + size_t(cr + 1) * kCand)) +
             "\n";
    for (int cr = 0; cr < kClasses; ++cr)
        o += "tailcls " + std::to_string(cr) + " " +
             dense(std::vector<uint64_t>(c.tail_cls.begin() + size_t(cr) * kCand,
                                         c.tail_cls.begin() + size_t(cr + 1) * kCand)) +
             "\n";
    o += "tailagg " + dense(c.tail_agg) + "\n";
    write_durably(path, o);
}

// ---- the gap state ----------------------------------------------------------

struct GapCampaign {
    GapTotals g;
    uint64_t evens = 0, walked = 0;
    std::vector<std::pair<uint64_t, uint64_t>> covered;
};

GapCampaign load_gaps(const std::string &path)
{
    GapCampaign gc;
    std::string all;
    if (!read_file(path, all)) return gc;
    const auto bad = [&](const std::string &ln) {
        return std::runtime_error("stats: gap state " + path + " has a malformed record '" + ln.substr(0, 80) +
                                  "'; refusing to merge into it");
    };
    unsigned seen = 0;
    size_t pos = 0;
    while (pos < all.size()) {
        const size_t e = all.find('\n', pos);
        if (e == std::string::npos) break;  // a cut-off last line: "end" is then missing
        const std::string ln = all.substr(pos, e - pos);
        pos = e + 1;
        if (ln.empty() || ln[0] == '#') continue;
        const std::vector<std::string> f = fields(ln);
        const std::string &k = f[0];
        const size_t nf = f.size();
        const auto once = [&](unsigned bit) {
            if (seen & bit) throw bad(ln);
            seen |= bit;
        };
        bool ok = true;
        uint64_t a = 0, b = 0;
        if (k == "gaps_range" && nf == 3) {
            ok = parse_u64(f[1], a) && parse_u64(f[2], b) && a <= b;
            gc.covered.push_back({a, b});
            seen |= 1;
        } else if (k == "gaps_evens" && nf == 3) {
            once(2);
            ok = parse_u64(f[1], gc.evens) && parse_u64(f[2], gc.walked);
        } else if (k == "gaps" && nf == 3) {
            once(4);
            ok = parse_u64(f[1], gc.g.n) && parse_u128(f[2], gc.g.d1);
        } else if (k == "gaps_samp" && nf <= 2) {
            once(8);
            ok = parse_dense(nf == 2 ? f[1] : std::string(), kGapHistBins, gc.g.samp);
        } else if (k == "gaps_max" && nf == 4) {
            once(16);
            ok = parse_u64(f[1], a) && parse_u64(f[2], b) && (f[3] == "0" || f[3] == "1");
            gc.g.gmax = a;
            gc.g.gmax_lo = b;
            // exactness below the tail is kept as "every range walked"
            gc.g.all_walked = f[3] == "1" && a < kGapTailMin;
        } else if (k == "gaps_walk" && nf == 6) {
            once(64);
            ok = parse_u64(f[1], gc.g.wn);
            for (int i = 0; i < 4 && ok; ++i) ok = parse_u128(f[2 + size_t(i)], gc.g.wd[i]);
        } else if (k == "gaps_tail" && nf == 4) {
            uint32_t g = 0;
            ok = parse_u32(f[1], g) && parse_u64(f[2], a) && parse_u64(f[3], b);
            if (ok) gc.g.note_tail(g, a, b);
        } else if (k == "end" && nf == 1) {
            once(32);
        } else {
            ok = false;
        }
        if (!ok) throw bad(ln);
    }
    if (seen != 127)
        throw std::runtime_error("stats: gap state " + path +
                                 " is cut off or missing records; refusing to merge into it");
    merge_ranges(gc.covered);
    return gc;
}

std::string gap_fields(const RunRecord &r)
{
    const GapTotals &g = r.gaps;
    std::string o = " gaps=" + std::to_string(g.n) + " gd1=" + u128_str(g.d1) + " gmax=" +
                    (g.gmax_exact() && g.gmax ? std::to_string(g.gmax) + ":" + std::to_string(g.gmax_lo) : "-") +
                    " gtail=";
    std::string t;
    for (const auto &e : g.tail)
        t += (t.empty() ? "" : ";") + std::to_string(e.first) + ":" + std::to_string(e.second.first) + ":" +
             std::to_string(e.second.second);
    o += t.empty() ? "-" : t;
    o += " gwalk=" + std::to_string(r.walk_evens) + ":" + std::to_string(g.wn) + " gsmom=";
    for (int k = 0; k < 4; ++k) o += (k ? "," : "") + u128_str(g.wd[k]);
    const std::string h = dense(g.samp);
    return o + " gsamp=" + (h.empty() ? std::string("-") : h);
}

// merges the run's gaps into the gap state (before the main state is
// written); false when the run's range is already in it
bool commit_gaps(const std::string &path, const RunRecord &r)
{
    GapCampaign gc = load_gaps(path);
    for (const auto &c : gc.covered)
        if (r.start <= c.second && c.first <= r.limit) {
            std::fprintf(stderr, "stats: gaps of [%llu, %llu] already in %s -- not recorded again\n",
                         (unsigned long long)r.start, (unsigned long long)r.limit, path.c_str());
            return false;
        }
    gc.g.merge(r.gaps);
    gc.evens += r.evens;
    gc.walked += r.walk_evens;
    gc.covered.push_back({r.start, r.limit});
    merge_ranges(gc.covered);
    std::string o =
        "# goldbach-l0 prime gap state v1 (exact; include/gstats.hpp GapStats)\n"
        "# gaps_range: lo hi with prime gaps recorded (upper prime in [lo + 1, hi - 1]);\n"
        "# gaps_evens <evens> <walked evens>; gaps <count> <sum g> (exact);\n"
        "# gaps_walk <count> <sum g> <sum g^2> <sum g^3> <sum g^4> and gaps_samp (histogram by g / 2): walked "
        "segments;\n"
        "# gaps_max <g> <lower> <1: exact, 0: largest seen>; gaps_tail <g> <count> <first lower> (g >= 700, "
        "exact)\n";
    for (const auto &c : gc.covered) o += "gaps_range " + std::to_string(c.first) + " " + std::to_string(c.second) + "\n";
    o += "gaps_evens " + std::to_string(gc.evens) + " " + std::to_string(gc.walked) + "\n";
    o += "gaps " + std::to_string(gc.g.n) + " " + u128_str(gc.g.d1) + "\ngaps_walk " + std::to_string(gc.g.wn);
    for (int k = 0; k < 4; ++k) o += " " + u128_str(gc.g.wd[k]);
    o += "\ngaps_samp " + dense(gc.g.samp) + "\n";
    o += "gaps_max " + std::to_string(gc.g.gmax) + " " + std::to_string(gc.g.gmax_lo) + " " +
         (gc.g.gmax_exact() ? "1" : "0") + "\n";
    for (const auto &t : gc.g.tail)
        o += "gaps_tail " + std::to_string(t.first) + " " + std::to_string(t.second.first) + " " +
             std::to_string(t.second.second) + "\n";
    o += "end\n";
    write_durably(path, o);
    return true;
}

bool gaps_cover(const std::string &path, uint64_t a, uint64_t b)
{
    for (const auto &c : load_gaps(path).covered)
        if (c.first <= a && b <= c.second) return true;
    return false;
}

// a log line with gap fields (a GBGAPS row or a GBSTATS line with gaps) for evens in [a, b]
bool log_has_gaps_in(const std::string &path, uint64_t a, uint64_t b)
{
    std::ifstream in(path, std::ios::binary);
    std::string ln;
    while (std::getline(in, ln)) {
        if (ln.compare(0, 2, "GB") != 0 || ln.find(" gd1=") == std::string::npos) continue;
        const size_t s = ln.find(" start="), l = ln.find(" limit=");
        if (s == std::string::npos || l == std::string::npos) continue;
        if (std::strtoull(ln.c_str() + s + 7, nullptr, 10) <= b && a <= std::strtoull(ln.c_str() + l + 7, nullptr, 10))
            return true;
    }
    return false;
}

}  // namespace

// ---- GapTotals, RunRecord ----------------------------------------------------

void GapTotals::note_max(uint64_t g, uint64_t lower)
{
    if (g > gmax || (g == gmax && g && lower < gmax_lo)) {
        gmax = g;
        gmax_lo = lower;
    }
}

void GapTotals::note_tail(uint32_t g, uint64_t count, uint64_t lower)
{
    auto &t = tail[g];
    if (!t.first || lower < t.second) t.second = lower;
    t.first += count;
}

void GapTotals::merge(const GapTotals &o)
{
    n += o.n;
    d1 += o.d1;
    for (const auto &t : o.tail) note_tail(t.first, t.second.first, t.second.second);
    note_max(o.gmax, o.gmax_lo);
    all_walked = all_walked && o.all_walked;
    wn += o.wn;
    for (int k = 0; k < 4; ++k) wd[k] += o.wd[k];
    for (size_t i = 0; i < samp.size(); ++i) samp[i] += o.samp[i];
}

uint64_t RunRecord::primes() const
{
    uint64_t s = 0;
    for (uint64_t v : primes30) s += v;
    return s;
}

uint64_t RunRecord::twins() const { return twins30[0] + twins30[1] + twins30[2]; }

uint64_t RunRecord::tail_evens() const
{
    uint64_t t = beyond.size();
    for (uint64_t v : tail_cls) t += v;
    for (uint64_t v : tail_agg) t += v;
    return t;
}

uint64_t RunRecord::pmax() const
{
    uint64_t m = 0;
    for (const auto &b : beyond) m = std::max(m, b.second);
    if (m) return m;
    const auto &cand = cands();
    for (int i = kCand - 1; i >= 0; --i) {
        bool any = tail_agg[size_t(i)] != 0;
        for (int cr = 0; cr < kClasses && !any; ++cr) any = tail_cls[size_t(cr) * kCand + size_t(i)] != 0;
        if (any) return cand[size_t(i)];
    }
    return 0;
}

std::string gbstats_line(const RunRecord &r, const std::vector<uint64_t> &camp_first, const std::string &version)
{
    const auto &cand = cands();
    std::string o = "GBSTATS v2 version=" + version;
    o += " start=" + std::to_string(r.start) + " limit=" + std::to_string(r.limit) + " evens=" +
         std::to_string(r.evens) + " evens_sampled=" + std::to_string(r.evens_sampled) + " tail_t=" +
         std::to_string(r.tail_t) + " tail_evens=" + std::to_string(r.tail_evens()) + " pmax=" +
         std::to_string(r.pmax()) + " primes=" + std::to_string(r.primes()) + " twins=" + std::to_string(r.twins());
    o += " primes30=";
    for (int i = 0; i < 8; ++i) o += (i ? "," : "") + std::to_string(r.primes30[i]);
    o += " twins30=";
    for (int i = 0; i < 3; ++i) o += (i ? "," : "") + std::to_string(r.twins30[i]);
    std::string nf;
    for (int i = 0; i < kCand; ++i) {
        const uint64_t f = r.first[size_t(i)], c = camp_first[size_t(i)];
        if (f && (!c || f < c)) nf += (nf.empty() ? "" : ";") + std::to_string(cand[size_t(i)]) + ":" + std::to_string(f);
    }
    o += " new_first=" + (nf.empty() ? std::string("-") : nf);
    std::string bey;
    for (const auto &b : r.beyond)
        bey += (bey.empty() ? "" : ";") + std::to_string(b.second) + ":" + std::to_string(b.first);
    o += " beyond=" + (bey.empty() ? std::string("-") : bey);
    if (r.gaps_on) o += gap_fields(r);
    // the tail by consecutive candidates from the first one >= tail_t, classes summed
    size_t t0 = 0;
    while (t0 < cand.size() && cand[t0] < r.tail_t) ++t0;
    std::vector<uint64_t> tot(kCand, 0);
    for (int i = 0; i < kCand; ++i) {
        tot[size_t(i)] = r.tail_agg[size_t(i)];
        for (int cr = 0; cr < kClasses; ++cr) tot[size_t(i)] += r.tail_cls[size_t(cr) * kCand + size_t(i)];
    }
    const std::string tl = t0 < cand.size() ? dense(tot, t0) : std::string();
    o += " tail=" + (tl.empty() ? std::string("-") : std::to_string(cand[t0]) + ":" + tl) + "\n";
    return o;
}

// ---- StatsCampaign -------------------------------------------------------------

StatsCampaign::StatsCampaign(std::string state_path, std::string log_path, std::string version, uint32_t tail_t)
    : state_path_(std::move(state_path)), log_path_(std::move(log_path)), version_(std::move(version)), tail_t_(tail_t)
{
}

void StatsCampaign::check() const
{
    (void)load_state(state_path_, tail_t_);
    (void)load_gaps(state_path_ + ".gaps");
}

std::string StatsCampaign::line(const RunRecord &r) const
{
    return gbstats_line(r, load_state(state_path_, tail_t_).first, version_);
}

std::string StatsCampaign::commit(const RunRecord &r, bool *merged)
{
    if (merged) *merged = false;
    if (r.tail_t != tail_t_)
        throw std::runtime_error("stats: the run's tail bound differs from the campaign's");
    const FileLock lock(state_path_ + ".lock");
    Campaign c = load_state(state_path_, tail_t_);
    const std::string gpath = state_path_ + ".gaps";
    for (const auto &cv : c.covered)
        if (r.start <= cv.second && cv.first <= r.limit) {
            std::fprintf(stderr,
                         "stats: [%llu, %llu] overlaps the covered range [%llu, %llu] of %s -- not recorded again\n",
                         (unsigned long long)r.start, (unsigned long long)r.limit, (unsigned long long)cv.first,
                         (unsigned long long)cv.second, state_path_.c_str());
            if (r.gaps_on) {
                // the run's p(n) sample as a row of its own; its gaps, when the
                // gap state does not hold them yet (a backfill)
                std::vector<uint64_t> ps(kCand, 0);
                for (int cr = 0; cr < kClasses; ++cr)
                    for (int i = 0; i < kCand; ++i) ps[size_t(i)] += r.samp[size_t(cr) * kCand + size_t(i)];
                append_log(log_path_, "GBPSAMP v1 version=" + version_ + " start=" + std::to_string(r.start) +
                                          " limit=" + std::to_string(r.limit) + " evens=" + std::to_string(r.evens) +
                                          " psev=" + std::to_string(r.evens_sampled) + " psamp=" + dense(ps) + "\n");
                const std::string row = "GBGAPS v1 version=" + version_ + " start=" + std::to_string(r.start) +
                                        " limit=" + std::to_string(r.limit) + " evens=" + std::to_string(r.evens) +
                                        gap_fields(r) + "\n";
                if (commit_gaps(gpath, r)) {
                    append_log(log_path_, row);
                } else if (gaps_cover(gpath, r.start, r.limit) && !log_has_gaps_in(log_path_, r.start, r.limit)) {
                    std::fprintf(stderr, "stats: %s has no gap row for [%llu, %llu] -- written now\n",
                                 log_path_.c_str(), (unsigned long long)r.start, (unsigned long long)r.limit);
                    append_log(log_path_, row);
                }
            }
            return gbstats_line(r, c.first, version_);
        }
    const std::string ln = gbstats_line(r, c.first, version_);
    for (size_t i = 0; i < c.samp.size(); ++i) {
        c.samp[i] += r.samp[i];
        c.tail_cls[i] += r.tail_cls[i];
    }
    for (int i = 0; i < kCand; ++i) {
        c.tail_agg[size_t(i)] += r.tail_agg[size_t(i)];
        const uint64_t f = r.first[size_t(i)];
        if (f && (!c.first[size_t(i)] || f < c.first[size_t(i)])) c.first[size_t(i)] = f;
    }
    for (int i = 0; i < 8; ++i) c.primes30[i] += r.primes30[i];
    for (int i = 0; i < 3; ++i) c.twins30[i] += r.twins30[i];
    c.evens += r.evens;
    c.sampled += r.evens_sampled;
    if (r.gaps_on) commit_gaps(gpath, r);
    c.beyond.insert(c.beyond.end(), r.beyond.begin(), r.beyond.end());
    c.covered.push_back({r.start, r.limit});
    merge_ranges(c.covered);
    save_state(state_path_, c, tail_t_);
    append_log(log_path_, ln);
    if (merged) *merged = true;
    return ln;
}

}  // namespace gb
