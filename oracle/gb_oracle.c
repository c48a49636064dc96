/*
 * gb_oracle.c -- CPU oracle of the dense Goldbach verify path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load or run this file, and only to verify
 * results or as the timed CPU baseline. The GPU product path (goldbach-l0_gb300/) never
 * links it and has no CPU fallback.
 *
 * What it restates (reference paths are relative to the goldbach-l0 project):
 *   - gbo_is_prime_u64: deterministic Miller-Rabin with the twelve bases
 *     2..37 after trial division by the same primes
 *     (src/primes.cpp:445-480).
 *   - gbo_min_goldbach_prime: the CPU fallback's witness search, ascending
 *     odd candidates <= 9781 and then every odd p beyond
 *     (src/primes.cpp:482-493; tests/stats_ref.cpp:80-84).
 *   - gbo_stats_line in MR mode: tests/stats_ref.cpp:64-190, the same fields
 *     in the same format (evens pmax primes twins primes30 twins30 first hist
 *     gaps gmom gmax gtail ghist).
 *   - Sieve mode computes the same line from an exact segmented sieve of
 *     Eratosthenes instead of per-number Miller-Rabin. It is cross-checked
 *     against MR mode on every window small enough for both, and it is
 *     what makes a whole 467.5M-integer segment at 4e18 checkable in
 *     seconds.
 *   - gbo_map_hash: the class-map hash of the GPU path. It is defined here
 *     because the reference has none: the sum mod 2^64 of splitmix64(q) over
 *     every prime q in [a, b] with gcd(q, 30) = 1, i.e. over exactly the set
 *     bits of a mod-30 class map of that range.
 *
 * Parity pins: tests/test_oracle.py checks this file against the fixtures in
 * tests/golden/ (stats_ref output and per-even p(n) of the compiled
 * reference, the published S(p) table, the base-2 pseudoprimes < 2^32).
 */
#define _GNU_SOURCE
#include <inttypes.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef unsigned __int128 u128;

#define GBO_MAX_CAND 9781u /* include/config.hpp:86 MAX_GB_PRIME */
#define GBO_NCAND_MAX 1300
#define GBO_GBINS 1024u /* gap histogram bins by g / 2 (g < 2048) */
#define GBO_GTAIL 700u  /* include/gstats.hpp:77 GAPS30_TAIL */
#define GBO_MAX_BEYOND 256

/* ------------------------------------------------------------------------ */
/* Candidate primes: the odd primes 3..9781 (include/config.hpp:81-86).      */
/* ------------------------------------------------------------------------ */
static uint16_t g_cand[GBO_NCAND_MAX];
static int g_ncand;
static int16_t g_cidx[GBO_MAX_CAND + 1]; /* p -> candidate index, -1 if none */
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

static void init_cands(void)
{
    static uint8_t comp[GBO_MAX_CAND + 1];
    memset(g_cidx, 0xFF, sizeof g_cidx);
    for (uint32_t i = 2; i * i <= GBO_MAX_CAND; ++i)
        if (!comp[i])
            for (uint32_t j = i * i; j <= GBO_MAX_CAND; j += i) comp[j] = 1;
    g_ncand = 0;
    for (uint32_t p = 3; p <= GBO_MAX_CAND; p += 2)
        if (!comp[p]) {
            g_cidx[p] = (int16_t)g_ncand;
            g_cand[g_ncand++] = (uint16_t)p;
        }
}

int gbo_num_candidates(void)
{
    pthread_once(&g_once, init_cands);
    return g_ncand;
}

int gbo_candidates(uint16_t *out, int cap)
{
    pthread_once(&g_once, init_cands);
    int n = g_ncand < cap ? g_ncand : cap;
    memcpy(out, g_cand, (size_t)n * sizeof(uint16_t));
    return n;
}

/* ------------------------------------------------------------------------ */
/* Deterministic Miller-Rabin (src/primes.cpp:445-480).                      */
/* ------------------------------------------------------------------------ */
static inline uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t n)
{
    return (uint64_t)(((u128)a * b) % n);
}

static inline uint64_t powmod64(uint64_t a, uint64_t e, uint64_t n)
{
    uint64_t r = 1;
    a %= n;
    while (e) {
        if (e & 1) r = mulmod64(r, a, n);
        a = mulmod64(a, a, n);
        e >>= 1;
    }
    return r;
}

int gbo_is_prime_u64(uint64_t n)
{
    static const uint64_t bases[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (n < 2) return 0;
    for (int i = 0; i < 12; ++i)
        if (n % bases[i] == 0) return n == bases[i];
    uint64_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) {
        d >>= 1;
        ++s;
    }
    for (int i = 0; i < 12; ++i) {
        uint64_t x = powmod64(bases[i], d, n);
        if (x == 1 || x == n - 1) continue;
        int composite = 1;
        for (int r = 1; r < s; ++r) {
            x = mulmod64(x, x, n);
            if (x == n - 1) {
                composite = 0;
                break;
            }
        }
        if (composite) return 0;
    }
    return 1;
}

/* src/primes.cpp:482-493 with cands = the odd primes <= 9781. */
uint64_t gbo_min_goldbach_prime(uint64_t n)
{
    pthread_once(&g_once, init_cands);
    if (n < 4 || (n & 1)) return 0;
    if (n == 4) return 2;
    for (int i = 0; i < g_ncand; ++i) {
        const uint64_t p = g_cand[i];
        if (p > n - p) return 0;
        if (gbo_is_prime_u64(n - p)) return p;
    }
    for (uint64_t p = (GBO_MAX_CAND + 1) | 1; p <= n / 2; p += 2)
        if (gbo_is_prime_u64(p) && gbo_is_prime_u64(n - p)) return p;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Exact odd-number sieve of [lo, hi] (lo, hi odd).                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    uint64_t lo, hi;  /* bit i <-> lo + 2 i */
    uint64_t nbits;
    uint64_t *w;      /* 1 = prime */
} oddmap;

static inline int om_get(const oddmap *m, uint64_t q)
{
    const uint64_t i = (q - m->lo) >> 1;
    return (int)((m->w[i >> 6] >> (i & 63)) & 1);
}

/* Odd primes <= n (n < 2^33), segmented, multithreaded. */
typedef struct {
    uint64_t n;
    const uint32_t *small;
    size_t nsmall;
    uint64_t blk0, blk1, blksz; /* odd index blocks [blk0, blk1) */
    uint32_t *out;
    size_t cnt, cap;
} bp_job;

static void *bp_worker(void *arg)
{
    bp_job *j = (bp_job *)arg;
    const uint64_t nodd = (j->n - 1) / 2; /* odd numbers 3..n: index i <-> 2i + 3 */
    uint8_t *buf = (uint8_t *)malloc(j->blksz);
    for (uint64_t b = j->blk0; b < j->blk1; ++b) {
        const uint64_t i0 = b * j->blksz;
        if (i0 >= nodd) break;
        const uint64_t i1 = i0 + j->blksz < nodd ? i0 + j->blksz : nodd;
        memset(buf, 1, (size_t)(i1 - i0));
        const uint64_t v0 = 2 * i0 + 3, v1 = 2 * (i1 - 1) + 3;
        for (size_t k = 0; k < j->nsmall; ++k) {
            const uint64_t p = j->small[k];
            if (p * p > v1) break;
            uint64_t s = p * p;
            if (s < v0) {
                s = ((v0 + p - 1) / p) * p;
                if (!(s & 1)) s += p;
            }
            for (uint64_t v = s; v <= v1; v += 2 * p) buf[(v - 3) / 2 - i0] = 0;
        }
        for (uint64_t i = i0; i < i1; ++i)
            if (buf[i - i0]) {
                if (j->cnt == j->cap) {
                    j->cap = j->cap ? 2 * j->cap : 1 << 20;
                    j->out = (uint32_t *)realloc(j->out, j->cap * sizeof(uint32_t));
                }
                j->out[j->cnt++] = (uint32_t)(2 * i + 3);
            }
    }
    free(buf);
    return NULL;
}

static int default_threads(void)
{
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

/* The odd primes <= n, ascending (n <= 2^32 - 1). Caller frees. */
uint32_t *gbo_odd_primes_upto(uint64_t n, size_t *count, int threads)
{
    if (threads <= 0) threads = default_threads();
    *count = 0;
    if (n < 3) return (uint32_t *)malloc(sizeof(uint32_t));
    /* primes up to sqrt(n) by a flat sieve */
    uint64_t r = 1;
    while ((r + 1) * (r + 1) <= n) ++r;
    uint8_t *c = (uint8_t *)calloc(r + 1, 1);
    uint32_t *small = (uint32_t *)malloc((r + 1) * sizeof(uint32_t));
    size_t ns = 0;
    for (uint64_t i = 2; i <= r; ++i)
        if (!c[i]) {
            if (i & 1) small[ns++] = (uint32_t)i;
            for (uint64_t k = i * i; k <= r; k += i) c[k] = 1;
        }
    free(c);
    const uint64_t nodd = (n - 1) / 2, blksz = 1 << 22;
    const uint64_t nblk = (nodd + blksz - 1) / blksz;
    if ((uint64_t)threads > nblk) threads = (int)(nblk ? nblk : 1);
    bp_job *jobs = (bp_job *)calloc((size_t)threads, sizeof(bp_job));
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) {
        jobs[t].n = n;
        jobs[t].small = small;
        jobs[t].nsmall = ns;
        jobs[t].blksz = blksz;
        jobs[t].blk0 = nblk * (uint64_t)t / (uint64_t)threads;
        jobs[t].blk1 = nblk * (uint64_t)(t + 1) / (uint64_t)threads;
        pthread_create(&th[t], NULL, bp_worker, &jobs[t]);
    }
    size_t tot = 0;
    for (int t = 0; t < threads; ++t) {
        pthread_join(th[t], NULL);
        tot += jobs[t].cnt;
    }
    uint32_t *out = (uint32_t *)malloc((tot ? tot : 1) * sizeof(uint32_t));
    size_t pos = 0;
    for (int t = 0; t < threads; ++t) {
        if (jobs[t].cnt) memcpy(out + pos, jobs[t].out, jobs[t].cnt * sizeof(uint32_t));
        pos += jobs[t].cnt;
        free(jobs[t].out);
    }
    free(jobs);
    free(th);
    free(small);
    *count = tot;
    return out;
}

static uint64_t isqrt64(uint64_t n)
{
    uint64_t r = 0;
    for (int b = 31; b >= 0; --b) {
        const uint64_t t = r | (1ull << b);
        if (t <= n / t) r = t;
    }
    return r;
}

typedef struct {
    oddmap *m;
    const uint32_t *pr;
    size_t npr;
    int tid, nth;
} sv_job;

static void *sv_worker(void *arg)
{
    sv_job *j = (sv_job *)arg;
    oddmap *m = j->m;
    for (size_t k = (size_t)j->tid; k < j->npr; k += (size_t)j->nth) {
        const uint64_t p = j->pr[k];
        if (p > m->hi / p) break;
        uint64_t s = p * p;
        if (s < m->lo) {
            s = (m->lo / p) * p;
            if (s < m->lo) s += p;
            if (!(s & 1)) s += p;
        }
        for (uint64_t v = s; v <= m->hi && v >= s; v += 2 * p) {
            const uint64_t i = (v - m->lo) >> 1;
            __atomic_fetch_and(&m->w[i >> 6], ~(1ull << (i & 63)), __ATOMIC_RELAXED);
            if (m->hi - v < 2 * p) break;
        }
    }
    return NULL;
}

/* Builds the exact primality map of the odd numbers in [lo, hi]. */
static int oddmap_build(oddmap *m, uint64_t lo, uint64_t hi, int threads)
{
    if (threads <= 0) threads = default_threads();
    if (!(lo & 1)) lo += 1;
    if (!(hi & 1)) hi -= 1;
    if (hi < lo) return -1;
    m->lo = lo;
    m->hi = hi;
    m->nbits = (hi - lo) / 2 + 1;
    const size_t nw = (size_t)((m->nbits + 63) / 64);
    m->w = (uint64_t *)malloc(nw * sizeof(uint64_t));
    if (!m->w) return -1;
    memset(m->w, 0xFF, nw * sizeof(uint64_t));
    if (m->nbits % 64) m->w[nw - 1] = (1ull << (m->nbits % 64)) - 1;
    if (lo == 1) m->w[0] &= ~1ull; /* 1 is not prime */
    size_t npr = 0;
    uint32_t *pr = gbo_odd_primes_upto(isqrt64(hi) + 1, &npr, threads);
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    sv_job *jobs = (sv_job *)calloc((size_t)threads, sizeof(sv_job));
    for (int t = 0; t < threads; ++t) {
        jobs[t] = (sv_job){m, pr, npr, t, threads};
        pthread_create(&th[t], NULL, sv_worker, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
    free(pr);
    return 0;
}

static void oddmap_free(oddmap *m)
{
    free(m->w);
    m->w = NULL;
}

/* ------------------------------------------------------------------------ */
/* Run statistics (tests/stats_ref.cpp:64-190).                             */
/* ------------------------------------------------------------------------ */
typedef struct {
    uint64_t evens;
    uint64_t hist[GBO_NCAND_MAX];
    uint64_t first[GBO_NCAND_MAX]; /* 0 = none */
    int nbeyond;                   /* p(n) > 9781 (or 0: counterexample) */
    uint64_t bp[GBO_MAX_BEYOND], bcount[GBO_MAX_BEYOND], bfirst[GBO_MAX_BEYOND];
    uint64_t primes30[30], twins30[30];
    /* gaps q - prev(q) for primes q in [start + 1, limit - 1] */
    uint64_t gaps;
    u128 gmom[4];
    uint64_t gmax, gmax_lo;
    uint64_t ghist[GBO_GBINS];
    uint64_t gtail_cnt[GBO_GBINS], gtail_lo[GBO_GBINS];
    int gap_overflow;
} gbo_stats;

static void st_add_pn(gbo_stats *s, uint64_t n, uint64_t p)
{
    if (p <= GBO_MAX_CAND && p >= 3 && g_cidx[p] >= 0) {
        const int i = g_cidx[p];
        s->hist[i]++;
        if (!s->first[i] || n < s->first[i]) s->first[i] = n;
        return;
    }
    for (int b = 0; b < s->nbeyond; ++b)
        if (s->bp[b] == p) {
            s->bcount[b]++;
            if (n < s->bfirst[b]) s->bfirst[b] = n;
            return;
        }
    if (s->nbeyond < GBO_MAX_BEYOND) {
        s->bp[s->nbeyond] = p;
        s->bcount[s->nbeyond] = 1;
        s->bfirst[s->nbeyond] = n;
        s->nbeyond++;
    }
}

static void st_add_gap(gbo_stats *s, uint64_t g, uint64_t up)
{
    s->gaps++;
    const u128 g1 = g, g2 = g1 * g1;
    s->gmom[0] += g1;
    s->gmom[1] += g2;
    s->gmom[2] += g2 * g1;
    s->gmom[3] += g2 * g2;
    if (g / 2 >= GBO_GBINS) {
        s->gap_overflow = 1;
    } else if (!(g & 1)) { /* stats_ref's histogram lists even gaps only (3 - 2 = 1 is not in it) */
        s->ghist[g / 2]++;
        if (g >= GBO_GTAIL) {
            if (!s->gtail_cnt[g / 2] || up - g < s->gtail_lo[g / 2]) s->gtail_lo[g / 2] = up - g;
            s->gtail_cnt[g / 2]++;
        }
    }
    if (g > s->gmax || (g == s->gmax && up - g < s->gmax_lo)) {
        s->gmax = g;
        s->gmax_lo = up - g;
    }
}

static void st_merge(gbo_stats *d, const gbo_stats *s)
{
    for (int i = 0; i < GBO_NCAND_MAX; ++i) {
        d->hist[i] += s->hist[i];
        if (s->first[i] && (!d->first[i] || s->first[i] < d->first[i])) d->first[i] = s->first[i];
    }
    for (int b = 0; b < s->nbeyond; ++b)
        for (uint64_t k = 0; k < s->bcount[b]; ++k) st_add_pn(d, s->bfirst[b], s->bp[b]);
    for (int i = 0; i < 30; ++i) {
        d->primes30[i] += s->primes30[i];
        d->twins30[i] += s->twins30[i];
    }
}

static void u128_str(u128 v, char *o)
{
    char t[48];
    int n = 0;
    do {
        t[n++] = (char)('0' + (int)(v % 10));
        v /= 10;
    } while (v);
    for (int i = 0; i < n; ++i) o[i] = t[n - 1 - i];
    o[n] = 0;
}

/* Appends with bounds; returns 0 on overflow. */
typedef struct {
    char *b;
    size_t cap, len;
    int ok;
} sbuf;

static void sb_printf(sbuf *s, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
#include <stdarg.h>
static void sb_printf(sbuf *s, const char *fmt, ...)
{
    if (!s->ok) return;
    va_list ap;
    va_start(ap, fmt);
    const int n = vsnprintf(s->b + s->len, s->cap - s->len, fmt, ap);
    va_end(ap);
    if (n < 0 || (size_t)n >= s->cap - s->len) {
        s->ok = 0;
        return;
    }
    s->len += (size_t)n;
}

/* The stats_ref output line (tests/stats_ref.cpp:97-189). */
static int st_format(const gbo_stats *s, char *buf, size_t cap)
{
    sbuf o = {buf, cap, 0, 1};
    uint64_t pmax = 0;
    for (int i = 0; i < g_ncand; ++i)
        if (s->hist[i]) pmax = g_cand[i];
    for (int b = 0; b < s->nbeyond; ++b)
        if (s->bp[b] > pmax) pmax = s->bp[b];
    uint64_t np = 0, ntw = 0;
    for (int i = 0; i < 30; ++i) {
        np += s->primes30[i];
        ntw += s->twins30[i];
    }
    sb_printf(&o, "evens=%" PRIu64 " pmax=%" PRIu64 " primes=%" PRIu64 " twins=%" PRIu64 " primes30=", s->evens,
              pmax, np, ntw);
    static const int u[8] = {1, 7, 11, 13, 17, 19, 23, 29};
    for (int i = 0; i < 8; ++i) sb_printf(&o, "%s%" PRIu64, i ? "," : "", s->primes30[u[i]]);
    sb_printf(&o, " twins30=%" PRIu64 ",%" PRIu64 ",%" PRIu64, s->twins30[11], s->twins30[17], s->twins30[29]);
    sb_printf(&o, " first=");
    /* every p with a count, ascending (candidates, then the ones beyond) */
    int f1 = 1;
    uint64_t bsorted[GBO_MAX_BEYOND];
    int nb = s->nbeyond;
    for (int b = 0; b < nb; ++b) bsorted[b] = (uint64_t)b;
    for (int a = 0; a < nb; ++a)
        for (int b = a + 1; b < nb; ++b)
            if (s->bp[bsorted[b]] < s->bp[bsorted[a]]) {
                uint64_t t = bsorted[a];
                bsorted[a] = bsorted[b];
                bsorted[b] = t;
            }
    /* p = 0 (a counterexample) and p = 2 (n = 4) sort before the candidates */
    for (int b = 0; b < nb; ++b)
        if (s->bp[bsorted[b]] < 3) {
            sb_printf(&o, "%s%" PRIu64 ":%" PRIu64, f1 ? "" : ";", s->bp[bsorted[b]], s->bfirst[bsorted[b]]);
            f1 = 0;
        }
    for (int i = 0; i < g_ncand; ++i)
        if (s->hist[i]) {
            sb_printf(&o, "%s%u:%" PRIu64, f1 ? "" : ";", g_cand[i], s->first[i]);
            f1 = 0;
        }
    for (int b = 0; b < nb; ++b)
        if (s->bp[bsorted[b]] > GBO_MAX_CAND) {
            sb_printf(&o, "%s%" PRIu64 ":%" PRIu64, f1 ? "" : ";", s->bp[bsorted[b]], s->bfirst[bsorted[b]]);
            f1 = 0;
        }
    sb_printf(&o, " hist=");
    int last = 0;
    for (int i = 0; i < g_ncand; ++i)
        if (s->hist[i]) last = i + 1;
    for (int i = 0; i < last; ++i) {
        if (i) sb_printf(&o, ",");
        if (s->hist[i]) sb_printf(&o, "%" PRIu64, s->hist[i]);
    }
    char m0[48], m1[48], m2[48], m3[48];
    u128_str(s->gmom[0], m0);
    u128_str(s->gmom[1], m1);
    u128_str(s->gmom[2], m2);
    u128_str(s->gmom[3], m3);
    sb_printf(&o, " gaps=%" PRIu64 " gmom=%s,%s,%s,%s gmax=%" PRIu64 ":%" PRIu64 " gtail=", s->gaps, m0, m1, m2, m3,
              s->gmax, s->gmax_lo);
    int t1 = 1;
    for (uint32_t b = GBO_GTAIL / 2; b < GBO_GBINS; ++b)
        if (s->gtail_cnt[b]) {
            sb_printf(&o, "%s%u:%" PRIu64 ":%" PRIu64, t1 ? "" : ";", 2 * b, s->gtail_cnt[b], s->gtail_lo[b]);
            t1 = 0;
        }
    if (t1) sb_printf(&o, "-");
    sb_printf(&o, " ghist=");
    uint32_t hb = 0;
    for (uint32_t b = 0; b < GBO_GBINS; ++b)
        if (s->ghist[b]) hb = b + 1;
    for (uint32_t b = 0; b < hb; ++b) {
        if (b) sb_printf(&o, ",");
        if (s->ghist[b]) sb_printf(&o, "%" PRIu64, s->ghist[b]);
    }
    return o.ok && !s->gap_overflow ? 0 : -1;
}

/* ---- MR mode (tests/stats_ref.cpp:72-95, 121-170) ----------------------- */
typedef struct {
    uint64_t start, limit, evens;
    int tid, nth;
    gbo_stats *st;
    /* gaps: this thread's chunk of [qlo, qhi] */
    uint64_t qa, qe, gfirst, glast;
    gbo_stats *gs;
} mr_job;

static void *mr_worker(void *arg)
{
    mr_job *j = (mr_job *)arg;
    gbo_stats *a = j->st;
    for (uint64_t i = (uint64_t)j->tid; i < j->evens; i += (uint64_t)j->nth) {
        const uint64_t n = j->start + 2 * i;
        st_add_pn(a, n, gbo_min_goldbach_prime(n));
        const uint64_t q = n + 1;
        if (q < j->limit && gbo_is_prime_u64(q)) {
            a->primes30[q % 30]++;
            if (q + 2 < j->limit && gbo_is_prime_u64(q + 2)) a->twins30[q % 30]++;
        }
    }
    for (uint64_t q = j->qa; q < j->qe; q += 2) {
        if (!gbo_is_prime_u64(q)) continue;
        if (j->glast) st_add_gap(j->gs, q - j->glast, q);
        else j->gfirst = q;
        j->glast = q;
    }
    return NULL;
}

static void gaps_merge(gbo_stats *G, const gbo_stats *c)
{
    G->gaps += c->gaps;
    for (int k = 0; k < 4; ++k) G->gmom[k] += c->gmom[k];
    for (uint32_t b = 0; b < GBO_GBINS; ++b) {
        G->ghist[b] += c->ghist[b];
        if (c->gtail_cnt[b]) {
            if (!G->gtail_cnt[b] || c->gtail_lo[b] < G->gtail_lo[b]) G->gtail_lo[b] = c->gtail_lo[b];
            G->gtail_cnt[b] += c->gtail_cnt[b];
        }
    }
    if (c->gmax > G->gmax || (c->gmax == G->gmax && c->gmax && c->gmax_lo < G->gmax_lo)) {
        G->gmax = c->gmax;
        G->gmax_lo = c->gmax_lo;
    }
    G->gap_overflow |= c->gap_overflow;
}

static int stats_mr(uint64_t start, uint64_t limit, int threads, gbo_stats *out)
{
    if (threads <= 0) threads = default_threads();
    const uint64_t evens = (limit - start) / 2 + 1;
    mr_job *jobs = (mr_job *)calloc((size_t)threads, sizeof(mr_job));
    gbo_stats *st = (gbo_stats *)calloc((size_t)threads, sizeof(gbo_stats));
    gbo_stats *gs = (gbo_stats *)calloc((size_t)threads, sizeof(gbo_stats));
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    const uint64_t qlo = start + 1, qhi = limit - 1;
    const uint64_t span = qhi >= qlo ? (qhi - qlo) / 2 + 1 : 0;
    for (int t = 0; t < threads; ++t) {
        mr_job *j = &jobs[t];
        j->start = start;
        j->limit = limit;
        j->evens = evens;
        j->tid = t;
        j->nth = threads;
        j->st = &st[t];
        j->gs = &gs[t];
        j->qa = qlo + 2 * (uint64_t)((u128)span * (uint64_t)t / (uint64_t)threads);
        j->qe = qlo + 2 * (uint64_t)((u128)span * (uint64_t)(t + 1) / (uint64_t)threads);
        pthread_create(&th[t], NULL, mr_worker, j);
    }
    memset(out, 0, sizeof *out);
    out->evens = evens;
    uint64_t glast = 0;
    for (int t = 0; t < threads; ++t) {
        pthread_join(th[t], NULL);
        st_merge(out, &st[t]);
    }
    /* stitch the chunks in order (tests/stats_ref.cpp:146-170) */
    for (int t = 0; t < threads; ++t) {
        const mr_job *j = &jobs[t];
        if (!j->gfirst) continue;
        uint64_t prev = glast;
        if (!prev) {
            prev = j->gfirst - 2;
            while (!gbo_is_prime_u64(prev)) prev -= 2;
        }
        st_add_gap(out, j->gfirst - prev, j->gfirst);
        gaps_merge(out, &gs[t]);
        glast = j->glast;
    }
    free(jobs);
    free(st);
    free(gs);
    free(th);
    return 0;
}

/* ---- sieve mode: the same statistics from an exact sieve ---------------- */
typedef struct {
    const oddmap *m;
    uint64_t start, limit, e0, e1;
    gbo_stats *st;
    int needs_mr; /* an even left without a witness <= 9781 */
} pn_job;

static inline int om_isprime(const oddmap *m, uint64_t q)
{
    if (q >= m->lo && q <= m->hi) return om_get(m, q);
    return gbo_is_prime_u64(q);
}

static void *pn_worker(void *arg)
{
    pn_job *j = (pn_job *)arg;
    for (uint64_t i = j->e0; i < j->e1; ++i) {
        const uint64_t n = j->start + 2 * i;
        uint64_t p = 0;
        if (n == 4) p = 2;
        else {
            for (int c = 0; c < g_ncand; ++c) {
                const uint64_t cp = g_cand[c];
                if (cp > n - cp) break;
                if (om_isprime(j->m, n - cp)) {
                    p = cp;
                    break;
                }
            }
            if (!p) p = gbo_min_goldbach_prime(n);
        }
        st_add_pn(j->st, n, p);
        const uint64_t q = n + 1;
        if (q < j->limit && om_isprime(j->m, q)) {
            j->st->primes30[q % 30]++;
            if (q + 2 < j->limit && om_isprime(j->m, q + 2)) j->st->twins30[q % 30]++;
        }
    }
    return NULL;
}

static int stats_sieve(uint64_t start, uint64_t limit, int threads, gbo_stats *out)
{
    if (threads <= 0) threads = default_threads();
    pthread_once(&g_once, init_cands);
    const uint64_t evens = (limit - start) / 2 + 1;
    uint64_t lo = start > GBO_MAX_CAND + 2100 ? start - GBO_MAX_CAND - 2100 : 1;
    oddmap m;
    if (oddmap_build(&m, lo | 1, limit + 1, threads)) return -1;
    pn_job *jobs = (pn_job *)calloc((size_t)threads, sizeof(pn_job));
    gbo_stats *st = (gbo_stats *)calloc((size_t)threads, sizeof(gbo_stats));
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) {
        jobs[t].m = &m;
        jobs[t].start = start;
        jobs[t].limit = limit;
        jobs[t].e0 = evens * (uint64_t)t / (uint64_t)threads;
        jobs[t].e1 = evens * (uint64_t)(t + 1) / (uint64_t)threads;
        jobs[t].st = &st[t];
        pthread_create(&th[t], NULL, pn_worker, &jobs[t]);
    }
    memset(out, 0, sizeof *out);
    out->evens = evens;
    for (int t = 0; t < threads; ++t) {
        pthread_join(th[t], NULL);
        st_merge(out, &st[t]);
    }
    /* gaps: every prime q in [start + 1, limit - 1], in order */
    uint64_t prev = 0;
    for (uint64_t q = (start + 1) | 1; q + 1 <= limit; q += 2) {
        if (!om_get(&m, q)) continue;
        if (!prev) {
            prev = q - 2;
            while (!om_isprime(&m, prev)) prev -= 2;
        }
        st_add_gap(out, q - prev, q);
        prev = q;
    }
    oddmap_free(&m);
    free(jobs);
    free(st);
    free(th);
    return 0;
}

/* mode 0 = MR (stats_ref's algorithm), 1 = exact sieve. Returns 0 on success. */
int gbo_stats_line(uint64_t start, uint64_t limit, int mode, int threads, char *buf, size_t cap)
{
    pthread_once(&g_once, init_cands);
    if (start % 2 || limit % 2 || start < 6 || limit < start) return -2;
    gbo_stats *s = (gbo_stats *)calloc(1, sizeof(gbo_stats));
    int rc = mode ? stats_sieve(start, limit, threads, s) : stats_mr(start, limit, threads, s);
    if (!rc) rc = st_format(s, buf, cap);
    free(s);
    return rc;
}

/* p(n) of the evens start, start + 2, ..., start + 2 (count - 1) (u16; a
 * p(n) above 65535 cannot occur below 2^64 in practice and is stored as 0). */
typedef struct {
    uint64_t start, e0, e1;
    const oddmap *m;
    uint16_t *out;
} pr_job;

static void *pr_worker(void *arg)
{
    pr_job *j = (pr_job *)arg;
    for (uint64_t i = j->e0; i < j->e1; ++i) {
        const uint64_t n = j->start + 2 * i;
        uint64_t p = 0;
        if (j->m && n != 4) {
            for (int c = 0; c < g_ncand; ++c) {
                const uint64_t cp = g_cand[c];
                if (cp > n - cp) break;
                if (om_isprime(j->m, n - cp)) {
                    p = cp;
                    break;
                }
            }
        }
        if (!p) p = gbo_min_goldbach_prime(n);
        j->out[i] = p < 65536 ? (uint16_t)p : 0;
    }
    return NULL;
}

int gbo_pn_range(uint64_t start, uint64_t count, int mode, int threads, uint16_t *out)
{
    pthread_once(&g_once, init_cands);
    if (threads <= 0) threads = default_threads();
    if (start % 2 || start < 4 || !count) return -2;
    oddmap m;
    const oddmap *mp = NULL;
    if (mode) {
        const uint64_t lo = start > GBO_MAX_CAND + 8 ? start - GBO_MAX_CAND - 4 : 1;
        if (oddmap_build(&m, lo | 1, start + 2 * count, threads)) return -1;
        mp = &m;
    }
    pr_job *jobs = (pr_job *)calloc((size_t)threads, sizeof(pr_job));
    pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) {
        jobs[t] = (pr_job){start, count * (uint64_t)t / (uint64_t)threads,
                           count * (uint64_t)(t + 1) / (uint64_t)threads, mp, out};
        pthread_create(&th[t], NULL, pr_worker, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    if (mp) oddmap_free(&m);
    free(jobs);
    free(th);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Class-map hash and per-range counts (the GPU path's self-check values).   */
/* ------------------------------------------------------------------------ */
static inline uint64_t splitmix64(uint64_t q)
{
    uint64_t z = q + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t gbo_mix(uint64_t q) { return splitmix64(q); }

/* Sum mod 2^64 of splitmix64(q) over the primes q in [a, b] coprime to 30,
 * and (optionally) their count. */
int gbo_map_hash(uint64_t a, uint64_t b, int threads, uint64_t *hash, uint64_t *count)
{
    if (b < a) {
        *hash = 0;
        if (count) *count = 0;
        return 0;
    }
    oddmap m;
    if (oddmap_build(&m, a | 1, b, threads)) {
        *hash = 0;
        if (count) *count = 0;
        return 0;
    }
    uint64_t h = 0, c = 0;
    for (uint64_t i = 0; i < m.nbits; ++i)
        if ((m.w[i >> 6] >> (i & 63)) & 1) {
            const uint64_t q = m.lo + 2 * i;
            if (q % 3 && q % 5) {
                h += splitmix64(q);
                ++c;
            }
        }
    oddmap_free(&m);
    *hash = h;
    if (count) *count = c;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* CLI                                                                       */
/* ------------------------------------------------------------------------ */
#ifndef GBO_NO_MAIN
static void usage(void)
{
    fprintf(stderr,
            "usage: gb_oracle stats START LIMIT [mr|sieve] [THREADS]\n"
            "       gb_oracle pn START COUNT [mr|sieve] [THREADS]\n"
            "       gb_oracle hash A B [THREADS]\n"
            "       gb_oracle isprime N...\n");
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        usage();
        return 2;
    }
    if (!strcmp(argv[1], "stats") && argc >= 4) {
        const uint64_t s = strtoull(argv[2], NULL, 10), l = strtoull(argv[3], NULL, 10);
        const int mode = argc > 4 && !strcmp(argv[4], "sieve");
        const int th = argc > 5 ? atoi(argv[5]) : 0;
        char *buf = (char *)malloc(1 << 20);
        const int rc = gbo_stats_line(s, l, mode, th, buf, 1 << 20);
        if (rc) {
            fprintf(stderr, "gb_oracle: failed (%d)\n", rc);
            return 1;
        }
        puts(buf);
        free(buf);
        return 0;
    }
    if (!strcmp(argv[1], "pn") && argc >= 4) {
        const uint64_t s = strtoull(argv[2], NULL, 10), c = strtoull(argv[3], NULL, 10);
        const int mode = argc > 4 && !strcmp(argv[4], "sieve");
        const int th = argc > 5 ? atoi(argv[5]) : 0;
        uint16_t *o = (uint16_t *)malloc(c * sizeof(uint16_t));
        if (gbo_pn_range(s, c, mode, th, o)) return 1;
        for (uint64_t i = 0; i < c; ++i) printf("%" PRIu64 " %u\n", s + 2 * i, o[i]);
        free(o);
        return 0;
    }
    if (!strcmp(argv[1], "hash") && argc >= 4) {
        uint64_t h, c;
        gbo_map_hash(strtoull(argv[2], NULL, 10), strtoull(argv[3], NULL, 10), argc > 4 ? atoi(argv[4]) : 0, &h,
                     &c);
        printf("hash=%016" PRIx64 " primes=%" PRIu64 "\n", h, c);
        return 0;
    }
    if (!strcmp(argv[1], "isprime")) {
        for (int i = 2; i < argc; ++i) printf("%s %d\n", argv[i], gbo_is_prime_u64(strtoull(argv[i], NULL, 10)));
        return 0;
    }
    usage();
    return 2;
}
#endif
