/*
 * gs_synth.c -- seeded synthetic references and reads (see gpuseed_synth.h).
 *
 * Determinism across machines: all draws are 64-bit integer generators
 * (splitmix64 seeding xoshiro256**), probabilities are compared as 53-bit
 * integer thresholds, and the one transcendental needed (exp, for log-normal
 * read lengths) is a Taylor series after ln2 range reduction evaluated with
 * plain IEEE multiplies and adds (the file is compiled without FP
 * contraction).  Normal deviates use the Irwin-Hall sum of twelve uniforms.
 * Work is split into fixed chunks with their own seeds, so the thread count
 * does not change the bytes.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/gpuseed_synth.h"

typedef struct {
    uint64_t s[4];
} rng_t;

static inline uint64_t splitmix64(uint64_t *x)
{
    uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static void rng_seed(rng_t *r, uint64_t seed)
{
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) r->s[i] = splitmix64(&x);
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t rng_next(rng_t *r)
{
    uint64_t *s = r->s;
    uint64_t res = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return res;
}

/* uniform integer in [0, n) (n > 0) */
static inline uint64_t rng_below(rng_t *r, uint64_t n)
{
    return (uint64_t)(((unsigned __int128)rng_next(r) * n) >> 64);
}

static inline uint64_t prob_thr(double p)
{
    if (p <= 0) return 0;
    if (p >= 1) return 1ull << 53;
    return (uint64_t)(p * 9007199254740992.0);
}

static inline int rng_bern(rng_t *r, uint64_t thr) { return (rng_next(r) >> 11) < thr; }

static inline double rng_unit(rng_t *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* exp(x) for |x| < 700: x = k ln2 + t, Taylor series of exp(t), 2^k by ldexp */
static double det_exp(double x)
{
    const double ln2 = 0.6931471805599453;
    double kf = x / ln2;
    long k = (long)(kf < 0 ? kf - 0.5 : kf + 0.5);
    double t = x - (double)k * ln2;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i <= 18; i++) {
        term = term * t / (double)i;
        sum = sum + term;
    }
    return ldexp(sum, (int)k);
}

static inline uint8_t bg_base(uint64_t r16, uint64_t gc_thr15)
{
    /* 15 bits decide G/C vs A/T, bit 15 picks within the pair */
    uint64_t v = r16 & 0x7fff;
    int hi = (int)((r16 >> 15) & 1);
    if (v < gc_thr15) return hi ? 2 : 1;    /* G : C */
    return hi ? 3 : 0;                      /* T : A */
}

typedef struct {
    const gs_synth_ref_spec *sp;
    uint8_t *codes;
    uint64_t chunk, n_chunks;
    volatile uint64_t next;
} bg_job;

static void *bg_worker(void *arg)
{
    bg_job *j = (bg_job *)arg;
    uint64_t gc_thr = (uint64_t)(j->sp->gc * 32768.0 + 0.5);
    for (;;) {
        uint64_t c = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
        if (c >= j->n_chunks) break;
        rng_t r;
        rng_seed(&r, j->sp->seed ^ (0x51ed270b27d3e1a5ull * (c + 1)));
        uint64_t b = c * j->chunk, e = b + j->chunk;
        if (e > j->sp->length) e = j->sp->length;
        for (uint64_t i = b; i < e; i += 4) {
            uint64_t x = rng_next(&r);
            for (int q = 0; q < 4 && i + q < e; q++) j->codes[i + q] = bg_base(x >> (16 * q), gc_thr);
        }
    }
    return NULL;
}

static void copy_diverged(rng_t *r, uint8_t *dst, const uint8_t *src, uint64_t len, double div)
{
    uint64_t thr = prob_thr(div);
    for (uint64_t i = 0; i < len; i++) {
        uint8_t c = src[i];
        if (rng_bern(r, thr)) c = (uint8_t)((c + 1 + rng_below(r, 3)) & 3);
        dst[i] = c;
    }
}

int gs_synth_reference(const gs_synth_ref_spec *sp, uint8_t *codes, uint8_t *nmask, int n_threads)
{
    if (!sp || !codes || sp->length == 0) return -1;
    uint64_t n = sp->length;
    if (n_threads <= 0) n_threads = 8;
    bg_job job = {sp, codes, 1u << 20, (n + (1u << 20) - 1) >> 20, 0};
    pthread_t th[64];
    if (n_threads > 64) n_threads = 64;
    for (int t = 0; t < n_threads; t++) pthread_create(&th[t], NULL, bg_worker, &job);
    for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);

    rng_t r;
    rng_seed(&r, sp->seed ^ 0xa0761d6478bd642full);
    uint64_t gc_thr = (uint64_t)(sp->gc * 32768.0 + 0.5);
    /* repeat families: a random consensus, copies at random places */
    if (sp->fam_unit && sp->fam_unit < n) {
        uint8_t *cons = (uint8_t *)malloc(sp->fam_unit);
        if (!cons) return -4;
        for (uint32_t f = 0; f < sp->fam_count; f++) {
            for (uint32_t i = 0; i < sp->fam_unit; i++) cons[i] = bg_base(rng_next(&r), gc_thr);
            for (uint32_t c = 0; c < sp->fam_copies; c++) {
                uint64_t pos = rng_below(&r, n - sp->fam_unit);
                double div = sp->fam_div_min + (sp->fam_div_max - sp->fam_div_min) * rng_unit(&r);
                copy_diverged(&r, codes + pos, cons, sp->fam_unit, div);
            }
        }
        free(cons);
    }
    /* segmental duplications: copy a random segment elsewhere, diverged */
    if (sp->dup_frac > 0 && sp->dup_len_max > 0 && sp->dup_len_max < n / 2) {
        uint64_t target = (uint64_t)(sp->dup_frac * (double)n);
        uint64_t done = 0;
        uint8_t *tmp = (uint8_t *)malloc(sp->dup_len_max);
        if (!tmp) return -4;
        while (done < target) {
            uint64_t len = sp->dup_len_min + rng_below(&r, (uint64_t)(sp->dup_len_max - sp->dup_len_min) + 1);
            uint64_t src = rng_below(&r, n - len), dst = rng_below(&r, n - len);
            double div = sp->dup_div_min + (sp->dup_div_max - sp->dup_div_min) * rng_unit(&r);
            memcpy(tmp, codes + src, len);
            copy_diverged(&r, codes + dst, tmp, len, div);
            done += len;
        }
        free(tmp);
    }
    if (nmask) {
        memset(nmask, 0, n);
        if (sp->n_frac > 0 && sp->n_block_max > 0 && sp->n_block_max < n) {
            uint64_t target = (uint64_t)(sp->n_frac * (double)n), done = 0;
            while (done < target) {
                uint64_t len = sp->n_block_min + rng_below(&r, (uint64_t)(sp->n_block_max - sp->n_block_min) + 1);
                uint64_t pos = rng_below(&r, n - len);
                memset(nmask + pos, 1, len);
                done += len;
            }
        }
    }
    return 0;
}

static uint32_t max_len(const gs_synth_read_spec *sp)
{
    switch (sp->len_mode) {
    case GS_LEN_FIXED: return sp->len_fixed;
    case GS_LEN_CHOICE: {
        uint32_t m = 0;
        for (uint32_t i = 0; i < sp->n_choices && i < 8; i++) if (sp->len_choices[i] > m) m = sp->len_choices[i];
        return m;
    }
    default: return sp->len_max;
    }
}

uint64_t gs_synth_reads_capacity(const gs_synth_read_spec *sp)
{
    return (uint64_t)sp->n_reads * max_len(sp) + 64;
}

static uint32_t draw_len(const gs_synth_read_spec *sp, rng_t *r)
{
    switch (sp->len_mode) {
    case GS_LEN_FIXED: return sp->len_fixed;
    case GS_LEN_CHOICE: return sp->len_choices[rng_below(r, sp->n_choices ? sp->n_choices : 1)];
    case GS_LEN_UNIFORM: return sp->len_min + (uint32_t)rng_below(r, (uint64_t)(sp->len_max - sp->len_min) + 1);
    default: {
        double z = -6.0;
        for (int i = 0; i < 12; i++) z = z + rng_unit(r);
        double v = sp->ln_median * det_exp(sp->ln_sigma * z);
        if (v < sp->len_min) v = sp->len_min;
        if (v > sp->len_max) v = sp->len_max;
        return (uint32_t)v;
    }
    }
}

typedef struct {
    const uint8_t *codes, *nmask;
    uint64_t n;
    const gs_synth_read_spec *sp;
    char *seqs;
    uint64_t *offsets;
    uint32_t *lengths;
    uint32_t maxL;
    volatile uint32_t next;
} rd_job;

static const char ACGT[4] = {'A', 'C', 'G', 'T'};

static void *rd_worker(void *arg)
{
    rd_job *j = (rd_job *)arg;
    const gs_synth_read_spec *sp = j->sp;
    uint64_t sub_thr = prob_thr(sp->sub_rate), ind_thr = prob_thr(sp->indel_rate);
    uint64_t nrun_thr = prob_thr(sp->nrun_frac);
    uint32_t imax = sp->indel_max ? sp->indel_max : 1;
    for (;;) {
        uint32_t r0 = __atomic_fetch_add(&j->next, 256u, __ATOMIC_RELAXED);
        if (r0 >= sp->n_reads) break;
        uint32_t r1 = r0 + 256 < sp->n_reads ? r0 + 256 : sp->n_reads;
        for (uint32_t rd = r0; rd < r1; rd++) {
            rng_t r;
            rng_seed(&r, sp->seed ^ (0x9fb21c651e98df25ull * ((uint64_t)rd + 1)));
            uint32_t L = draw_len(sp, &r);
            char *out = j->seqs + (uint64_t)rd * j->maxL;
            j->offsets[rd] = (uint64_t)rd * j->maxL;
            j->lengths[rd] = L;
            /* source window long enough for deletions */
            uint64_t span = (uint64_t)L + 2 * imax * 8 + 16;
            if (span > j->n) span = j->n;
            uint64_t start = rng_below(&r, j->n - span + 1);
            int minus = (int)(rng_next(&r) & 1);
            uint64_t si = 0;
            for (uint32_t o = 0; o < L;) {
                if (si >= span) si = 0;   /* wrap inside the window (tiny references only) */
                uint64_t p = minus ? start + span - 1 - si : start + si;
                uint8_t c = j->codes[p];
                char ch = j->nmask && j->nmask[p] ? 'N' : ACGT[minus ? 3 - c : c];
                if (ind_thr && rng_bern(&r, ind_thr)) {
                    uint32_t il = 1 + (uint32_t)rng_below(&r, imax);
                    if (rng_next(&r) & 1) {
                        for (uint32_t q = 0; q < il && o < L; q++) out[o++] = ACGT[rng_below(&r, 4)];
                    } else {
                        si += il;
                    }
                    continue;
                }
                if (ch != 'N' && rng_bern(&r, sub_thr)) {
                    int cc = (ch == 'A') ? 0 : (ch == 'C') ? 1 : (ch == 'G') ? 2 : 3;
                    ch = ACGT[(cc + 1 + rng_below(&r, 3)) & 3];
                }
                out[o++] = ch;
                si++;
            }
            if (nrun_thr && rng_bern(&r, nrun_thr) && L > 0) {
                uint32_t nl = sp->nrun_min + (uint32_t)rng_below(&r, (uint64_t)(sp->nrun_max - sp->nrun_min) + 1);
                if (nl > L) nl = L;
                uint32_t at = (uint32_t)rng_below(&r, (uint64_t)(L - nl) + 1);
                memset(out + at, 'N', nl);
            }
        }
    }
    return NULL;
}

int gs_synth_reads(const uint8_t *codes, const uint8_t *nmask, uint64_t length,
                   const gs_synth_read_spec *sp, char *seqs, uint64_t seqs_cap,
                   uint64_t *offsets, uint32_t *lengths, int n_threads)
{
    if (!codes || !sp || !seqs || !offsets || !lengths || length == 0) return -1;
    uint32_t maxL = max_len(sp);
    if ((uint64_t)sp->n_reads * maxL > seqs_cap) return -7;
    if (n_threads <= 0) n_threads = 8;
    if (n_threads > 64) n_threads = 64;
    rd_job job = {codes, nmask, length, sp, seqs, offsets, lengths, maxL, 0};
    pthread_t th[64];
    for (int t = 0; t < n_threads; t++) pthread_create(&th[t], NULL, rd_worker, &job);
    for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
    /* pack the fixed-stride records back to back */
    uint64_t w = 0;
    for (uint32_t rd = 0; rd < sp->n_reads; rd++) {
        if (offsets[rd] != w) memmove(seqs + w, seqs + offsets[rd], lengths[rd]);
        offsets[rd] = w;
        w += lengths[rd];
    }
    return 0;
}
