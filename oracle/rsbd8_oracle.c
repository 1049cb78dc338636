/*
 * rsbd8_oracle.c - the ORACLE for the GB300 radix sort.
 *
 * Test infrastructure only: the parity tests, the smoke check and the CPU
 * baseline leg of bench.py call this code to verify results (or as the timed
 * CPU stand-in of the reference).  Nothing on the product path links it.
 *
 * It is a plain-C restatement of the stable LSD radix sort in
 * Radixsortbidi8.hpp (namespace rsbd8), following the reference's structure:
 *   - mode resolution: helper::isabsvalue / issignmode / isfltpmode /
 *     isdescsort / isrevorderwithindirection / isrevorderwithoutindirection
 *     (Radixsortbidi8.hpp:59778-59904);
 *   - the sort-key filter of each of the 8 filter combinations: filterinput
 *     (Radixsortbidi8.hpp:10006-10027) plus the virtual most-significant-bit
 *     flip of the signed and floating-point modes and the virtual
 *     least-significant-bit flip of tiered absolute floating-point, both
 *     applied by the offsets generators (Radixsortbidi8.hpp:11629-11806);
 *   - the digit geometry: typeradix / offsetsloopcount / typeradixremainder
 *     (Radixsortbidi8.hpp:1848-1869): 11-bit digits for 32- and 64-bit keys,
 *     8-bit digits for 8- and 16-bit keys;
 *   - one up-front histogram of every digit in one read of the keys
 *     (radixsortnoallocmultiinitmt, Radixsortbidi8.hpp:28919) and the
 *     pass-skip test "one bucket holds every key" (generateoffsets*,
 *     Radixsortbidi8.hpp:12238-12440, addcarryofless Radixsortbidi8.hpp:2903);
 *   - one stable scatter per surviving digit that always stores the original
 *     bits, recomputing the filtered digit from them each pass
 *     (radixsortnoallocmultisortmain, Radixsortbidi8.hpp:31782-31982; filtershift
 *     Radixsortbidi8.hpp:5592-5615);
 *   - indirection re-reads the key through the pointer on every pass
 *     (Radixsortbidi8.hpp:39977-39980) and moves only the pointers;
 *   - isrevorder is realised as a reversed read of the input in the first
 *     surviving pass (the reference makes a reversed copy in its histogram
 *     pass, Radixsortbidi8.hpp:28933-29088).
 * The reference's thread scheme (2-way bidirectional fill plus split/merge)
 * is replaced here by the textbook parallel LSD: per-thread slice counts,
 * per-thread bucket offsets, in-order scatter of each slice.  The result of
 * a stable LSD sort depends only on the key order and stability, so the
 * output is identical.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#include "rsbd8_oracle.h"

/* ---- mode resolution (Radixsortbidi8.hpp:59778-59904) ---------------- */

int rsbd8o_resolve(uint32_t kind, uint32_t mode, uint32_t direction, uint32_t indirect,
                   rsbd8o_desc *d)
{
    /* std::is_signed_v is true for signed integers and floating-point types,
     * false for unsigned integers, bool, enumerations and classes. */
    int is_signed = (kind == RSBD8O_KIND_SIGNED || kind == RSBD8O_KIND_FLOAT);
    int is_float = (kind == RSBD8O_KIND_FLOAT);
    if (!(mode < 8u || (mode >= 64u && mode <= 66u))) return -1;
    if (direction > 3u) return -1;
    d->absv = (mode >= 65u && is_signed) || (mode < 64u && (mode & 1u));
    d->sign = (mode >= 64u && mode <= 65u && is_signed) || (mode < 64u && (mode & 2u));
    d->fltp = (mode >= 64u && is_float) || (mode < 64u && (mode & 4u));
    d->desc = direction & 1u;
    d->indirect = indirect;
    if (indirect) {
        d->rev = (direction >> 1) & 1u;
    } else {
        /* reverse ordering is only honoured where distinct bit patterns can
         * share a sort key: both regular absolute modes and regular
         * floating-point (Radixsortbidi8.hpp:59877-59904) */
        d->rev = ((direction >> 1) & 1u) &&
                 ((d->absv && d->sign) || (!d->absv && d->sign && d->fltp));
    }
    return 0;
}

/* ---- sort key K(b) ---------------------------------------------------- */

/* Transform raw key bits b (width w bits, held in the low bits of a uint64)
 * into an unsigned sort key whose ascending order is the reference's
 * ascending order for the resolved mode.  Descending sorts use ~K. */
static inline uint64_t sortkey(uint64_t b, unsigned w, const rsbd8o_desc *d)
{
    const uint64_t mask = (w == 64u) ? ~(uint64_t)0 : (((uint64_t)1 << w) - 1u);
    const uint64_t sb = (uint64_t)1 << (w - 1u);
    const int s = (b & sb) != 0;
    const uint64_t m = b & ~sb;
    uint64_t k;
    if (d->absv != d->fltp) {               /* two-register filtering */
        if (d->absv) {                       /* integer absolute modes */
            if (d->sign) k = s ? ((0u - b) & mask) : b;            /* forceabssigned */
            else k = ((b << 1) & mask) ^ (s ? mask : 0u);         /* forcetieredabssigned */
        } else {                             /* floating-point, not absolute */
            if (d->sign) k = (s ? ((0u - m) & mask) : m) ^ sb;   /* forcefloatingp + MSB flip */
            else k = s ? (mask ^ m) : m;                          /* specialfloatingp */
        }
    } else if (d->absv) {                    /* absv && fltp: one-register filtering */
        if (d->sign) k = m;                                       /* forceabsfloatingp */
        else k = (((b << 1) & mask) | (b >> (w - 1u))) ^ 1u;    /* tiered abs float: rotl1 + LSB flip */
    } else {
        k = d->sign ? (b ^ sb) : b;                               /* forcesigned (MSB flip) / forceunsigned */
    }
    if (d->desc) k = ~k & mask;
    return k;
}

uint64_t rsbd8o_sortkey(uint64_t bits, uint32_t key_bytes, const rsbd8o_desc *d)
{
    return sortkey(bits, key_bytes * 8u, d);
}

/* ---- digit geometry (Radixsortbidi8.hpp:1848-1869) -------------------- */

static unsigned digit_bits(unsigned w) { return (w == 32u || w == 64u) ? 11u : 8u; }
static unsigned digit_count(unsigned w) { unsigned r = digit_bits(w); return (w + r - 1u) / r; }

/* ---- the parallel LSD engine ------------------------------------------ */

typedef struct sortjob {
    const rsbd8o_desc *d;
    unsigned w;             /* key width in bits */
    unsigned esize;         /* element size in bytes (key bytes, or 8 for pointers) */
    uint64_t n;
    const unsigned char *in;
    unsigned char *out, *buf;
    unsigned threads;
    pthread_barrier_t bar;
    uint64_t *counts;       /* threads x digits x buckets */
    uint64_t *totals;       /* digits x buckets */
    int skip[8];
    int ndig;
    /* per-pass state written by thread 0 */
    const unsigned char *src;
    unsigned char *dst;
    int reverse_src;
    unsigned shift, dbits;
} sortjob;

typedef struct worker { sortjob *j; unsigned t; } worker;

static inline uint64_t load_bits(const unsigned char *p, unsigned kb)
{
    switch (kb) {
    case 1: return *p;
    case 2: { uint16_t v; memcpy(&v, p, 2); return v; }
    case 4: { uint32_t v; memcpy(&v, p, 4); return v; }
    default: { uint64_t v; memcpy(&v, p, 8); return v; }
    }
}

/* raw key bits of element e (a key, or a pointer to the object holding it) */
static inline uint64_t elem_bits(const sortjob *j, const unsigned char *e)
{
    const unsigned kb = j->w / 8u;
    if (!j->d->indirect) return load_bits(e, kb);
    uintptr_t p; memcpy(&p, e, sizeof p);
    const unsigned char *obj = (const unsigned char *)p + j->d->offset1;
    if (j->d->indirect == 2) {
        uintptr_t q; memcpy(&q, obj, sizeof q);
        obj = (const unsigned char *)q + j->d->offset2;
    }
    return load_bits(obj, kb);
}

static void slice(uint64_t n, unsigned threads, unsigned t, uint64_t *lo, uint64_t *hi)
{
    *lo = n * t / threads;
    *hi = n * (t + 1u) / threads;
}

static void *work(void *arg)
{
    worker *wk = (worker *)arg;
    sortjob *j = wk->j;
    const unsigned t = wk->t, T = j->threads, es = j->esize;
    const unsigned nb = 1u << digit_bits(j->w);
    uint64_t lo, hi;
    slice(j->n, T, t, &lo, &hi);

    /* up-front histogram of every digit in one read of the keys */
    uint64_t *mine = j->counts + (uint64_t)t * 8u * nb;
    memset(mine, 0, sizeof(uint64_t) * 8u * nb);
    for (uint64_t i = lo; i < hi; ++i) {
        uint64_t k = sortkey(elem_bits(j, j->in + i * es), j->w, j->d);
        for (int g = 0; g < j->ndig; ++g) {
            unsigned sh = (unsigned)g * digit_bits(j->w);
            mine[(unsigned)g * nb + ((k >> sh) & (nb - 1u))]++;
        }
    }
    pthread_barrier_wait(&j->bar);
    if (t == 0) {
        memset(j->totals, 0, sizeof(uint64_t) * 8u * nb);
        for (unsigned u = 0; u < T; ++u)
            for (unsigned x = 0; x < 8u * nb; ++x) j->totals[x] += j->counts[(uint64_t)u * 8u * nb + x];
        for (int g = 0; g < j->ndig; ++g) {
            j->skip[g] = 0;
            for (unsigned x = 0; x < nb; ++x)
                if (j->totals[(unsigned)g * nb + x] == j->n) j->skip[g] = 1;
        }
    }
    pthread_barrier_wait(&j->bar);

    int k = 0;
    for (int g = 0; g < j->ndig; ++g) k += !j->skip[g];
    int i_pass = 0;
    const unsigned char *cur = j->in;
    for (int g = 0; g < j->ndig; ++g) {
        if (j->skip[g]) continue;
        ++i_pass;
        unsigned char *dst = ((k - i_pass) % 2 == 0) ? j->out : j->buf;
        const int rev = (i_pass == 1) && j->d->rev;
        const unsigned sh = (unsigned)g * digit_bits(j->w);
        /* slice counts of this digit over the current sequence */
        uint64_t *cnt = j->counts + (uint64_t)t * 8u * nb;
        memset(cnt, 0, sizeof(uint64_t) * nb);
        for (uint64_t i = lo; i < hi; ++i) {
            uint64_t src_i = rev ? (j->n - 1u - i) : i;
            uint64_t key = sortkey(elem_bits(j, cur + src_i * es), j->w, j->d);
            cnt[(key >> sh) & (nb - 1u)]++;
        }
        pthread_barrier_wait(&j->bar);
        /* offsets of this thread: bucket base + counts of earlier slices */
        uint64_t *off = (uint64_t *)malloc(sizeof(uint64_t) * nb);
        uint64_t run = 0;
        for (unsigned x = 0; x < nb; ++x) {
            uint64_t before = 0;
            for (unsigned u = 0; u < t; ++u) before += j->counts[(uint64_t)u * 8u * nb + x];
            off[x] = run + before;
            for (unsigned u = 0; u < T; ++u) run += j->counts[(uint64_t)u * 8u * nb + x];
        }
        for (uint64_t i = lo; i < hi; ++i) {
            uint64_t src_i = rev ? (j->n - 1u - i) : i;
            const unsigned char *e = cur + src_i * es;
            uint64_t key = sortkey(elem_bits(j, e), j->w, j->d);
            memcpy(dst + off[(key >> sh) & (nb - 1u)]++ * es, e, es);
        }
        free(off);
        pthread_barrier_wait(&j->bar);
        cur = dst;
    }
    if (k == 0) {   /* every digit skipped: plain (or reversed) copy */
        for (uint64_t i = lo; i < hi; ++i) {
            uint64_t src_i = j->d->rev ? (j->n - 1u - i) : i;
            memcpy(j->out + i * es, j->in + src_i * es, es);
        }
    }
    return NULL;
}

int rsbd8o_sortcopy(const rsbd8o_desc *d, uint64_t n, const void *in, void *out,
                    unsigned threads)
{
    if (d->key_bytes != 1 && d->key_bytes != 2 && d->key_bytes != 4 && d->key_bytes != 8) return -1;
    if (d->indirect > 2u) return -1;
    const unsigned es = d->indirect ? 8u : d->key_bytes;
    if (n == 0) return 0;
    if (n == 1) { memcpy(out, in, es); return 0; }
    if (threads == 0) threads = 1;
    if (threads > 256) threads = 256;
    if ((uint64_t)threads > n / 4096u + 1u) threads = (unsigned)(n / 4096u + 1u);

    sortjob j;
    memset(&j, 0, sizeof j);
    j.d = d; j.w = d->key_bytes * 8u; j.esize = es; j.n = n;
    j.in = (const unsigned char *)in; j.out = (unsigned char *)out;
    j.threads = threads; j.ndig = (int)digit_count(j.w);
    const unsigned nb = 1u << digit_bits(j.w);
    j.buf = (unsigned char *)malloc(n * es);
    j.counts = (uint64_t *)malloc(sizeof(uint64_t) * 8u * nb * threads);
    j.totals = (uint64_t *)malloc(sizeof(uint64_t) * 8u * nb);
    if (!j.buf || !j.counts || !j.totals) { free(j.buf); free(j.counts); free(j.totals); return -2; }
    pthread_barrier_init(&j.bar, NULL, threads);
    worker *wk = (worker *)malloc(sizeof(worker) * threads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    for (unsigned t = 0; t < threads; ++t) { wk[t].j = &j; wk[t].t = t; }
    for (unsigned t = 1; t < threads; ++t) pthread_create(&th[t], NULL, work, &wk[t]);
    work(&wk[0]);
    for (unsigned t = 1; t < threads; ++t) pthread_join(th[t], NULL);
    pthread_barrier_destroy(&j.bar);
    free(wk); free(th); free(j.buf); free(j.counts); free(j.totals);
    return 0;
}

/* ---- batches of independent sorts ------------------------------------- */
/* The reference has no batched entry point: its callers loop over radixsortcopy per array
 * (Radixsortbidi8.hpp:60476).  The oracle runs that loop with one sort per worker thread,
 * the workers taking the next job from a shared counter. */

typedef struct batchctl {
    uint64_t njobs;
    const rsbd8o_job *jobs;
    uint64_t next;          /* next job to take (guarded by mu) */
    int rc;
    pthread_mutex_t mu;
} batchctl;

static void *batch_work(void *arg)
{
    batchctl *b = (batchctl *)arg;
    for (;;) {
        pthread_mutex_lock(&b->mu);
        const uint64_t i = b->next++;
        pthread_mutex_unlock(&b->mu);
        if (i >= b->njobs) break;
        const rsbd8o_job *jb = &b->jobs[i];
        int rc = rsbd8o_sortcopy(jb->d, jb->n, jb->in, jb->out, 1);
        if (rc != 0) {
            pthread_mutex_lock(&b->mu);
            if (b->rc == 0) b->rc = rc;
            pthread_mutex_unlock(&b->mu);
        }
    }
    return NULL;
}

int rsbd8o_sortcopy_batch(uint64_t njobs, const rsbd8o_job *jobs, unsigned threads)
{
    if (njobs == 0) return 0;
    if (threads == 0) threads = 1;
    if (threads > 256) threads = 256;
    if ((uint64_t)threads > njobs) threads = (unsigned)njobs;
    batchctl b;
    b.njobs = njobs; b.jobs = jobs; b.next = 0; b.rc = 0;
    pthread_mutex_init(&b.mu, NULL);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    for (unsigned t = 1; t < threads; ++t) pthread_create(&th[t], NULL, batch_work, &b);
    batch_work(&b);
    for (unsigned t = 1; t < threads; ++t) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&b.mu);
    free(th);
    return b.rc;
}

/* which digits the reference's pass-skip test would drop (bit g = digit g) */
uint32_t rsbd8o_skipmask(const rsbd8o_desc *d, uint64_t n, const void *in, uint32_t digit_bits_override)
{
    const unsigned w = d->key_bytes * 8u;
    const unsigned db = digit_bits_override ? digit_bits_override : digit_bits(w);
    const unsigned nd = (w + db - 1u) / db, nb = 1u << db;
    uint64_t *h = (uint64_t *)calloc((size_t)nd * nb, sizeof(uint64_t));
    sortjob j; memset(&j, 0, sizeof j); j.d = d; j.w = w;
    const unsigned es = d->indirect ? 8u : d->key_bytes;
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t k = sortkey(elem_bits(&j, (const unsigned char *)in + i * es), w, d);
        for (unsigned g = 0; g < nd; ++g) h[g * nb + ((k >> (g * db)) & (nb - 1u))]++;
    }
    uint32_t mask = 0;
    for (unsigned g = 0; g < nd; ++g)
        for (unsigned x = 0; x < nb; ++x) if (h[g * nb + x] == n) mask |= 1u << g;
    free(h);
    return mask;
}
