/*
 * oracle.c -- CPU restatement of GPUseed's seeding path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Each function names the lines of
 * the reference file seed_gen.cu that it restates.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <errno.h>
#include <pthread.h>
#include <sched.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define OCC_INTERVAL 64u      /* seed_gen.cu:29 */
#define BLOCK_WORDS 8u        /* 4 counts + OCC_INTERVAL/16 words (:52-58) */
#define K0 13                 /* pre_calc_seed_len (seed_gen.cu:2822) */

enum { OR_OK = 0, OR_EIO = -2, OR_EFORMAT = -3, OR_ENOMEM = -4, OR_EINVAL = -5,
       OR_EWALK = -6 };

/* ------------------------------------------------------------------ */
/* index loading: bwt_restore_bwt / bwt_restore_sa (seed_gen.cu:2685-2736) */

static uint64_t expected_bwt_words(uint32_t seq_len)
{
    /* bwa's bwt_bwtupdate_core layout: a 4-word count block every 64 rows
     * plus a final count block, and one word per 16 rows. */
    uint64_t n_occ = ((uint64_t)seq_len + OCC_INTERVAL - 1) / OCC_INTERVAL + 1;
    return 4 * n_occ + ((uint64_t)seq_len + 15) / 16;
}

static int finish_index(or_index *idx)
{
    /* pad so that every 64-row block has its 4 BWT words addressable */
    uint64_t nblk = (uint64_t)idx->seq_len / OCC_INTERVAL + 2;
    uint64_t need = nblk * BLOCK_WORDS;
    if (idx->bwt_words < need) {
        uint32_t *p = (uint32_t *)realloc(idx->bwt, need * 4);
        if (!p) return OR_ENOMEM;
        memset(p + idx->bwt_words, 0, (need - idx->bwt_words) * 4);
        idx->bwt = p;
    }
    return OR_OK;
}

int or_index_load(const char *prefix, or_index **out)
{
    *out = NULL;
    size_t pl = strlen(prefix);
    char *fn = (char *)malloc(pl + 8);
    if (!fn) return OR_ENOMEM;
    or_index *idx = (or_index *)calloc(1, sizeof(or_index));
    if (!idx) { free(fn); return OR_ENOMEM; }
    int rc = OR_OK;

    /* .bwt: primary, L2[1..4], then the interleaved blocks (:2717-2736) */
    memcpy(fn, prefix, pl); strcpy(fn + pl, ".bwt");
    FILE *fp = fopen(fn, "rb");
    if (!fp) { rc = OR_EIO; goto fail; }
    fseek(fp, 0, SEEK_END);
    long fsz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    if (fsz < 20 || (fsz - 20) % 4) { fclose(fp); rc = OR_EFORMAT; goto fail; }
    idx->bwt_words = (uint64_t)(fsz - 20) / 4;
    if (fread(&idx->primary, 4, 1, fp) != 1 || fread(idx->L2 + 1, 4, 4, fp) != 4) {
        fclose(fp); rc = OR_EFORMAT; goto fail;
    }
    idx->L2[0] = 0;
    idx->seq_len = idx->L2[4];
    idx->bwt = (uint32_t *)malloc(idx->bwt_words * 4 + 64);
    if (!idx->bwt) { fclose(fp); rc = OR_ENOMEM; goto fail; }
    if (fread(idx->bwt, 4, idx->bwt_words, fp) != idx->bwt_words) {
        fclose(fp); rc = OR_EFORMAT; goto fail;
    }
    fclose(fp);
    if (idx->seq_len == 0 || idx->primary > idx->seq_len ||
        idx->L2[1] > idx->L2[2] || idx->L2[2] > idx->L2[3] || idx->L2[3] > idx->L2[4] ||
        idx->bwt_words < expected_bwt_words(idx->seq_len)) {
        rc = OR_EFORMAT; goto fail;
    }

    /* .sa: primary, 4 skipped words, sa_intv, seq_len, samples (:2685-2715) */
    strcpy(fn + pl, ".sa");
    fp = fopen(fn, "rb");
    if (!fp) { rc = OR_EIO; goto fail; }
    uint32_t hdr[7];
    if (fread(hdr, 4, 7, fp) != 7) { fclose(fp); rc = OR_EFORMAT; goto fail; }
    if (hdr[0] != idx->primary || hdr[6] != idx->seq_len || hdr[5] == 0) {
        fclose(fp); rc = OR_EFORMAT; goto fail;
    }
    idx->sa_intv = hdr[5];
    idx->n_sa = (uint32_t)(((uint64_t)idx->seq_len + idx->sa_intv) / idx->sa_intv);
    idx->sa = (uint32_t *)calloc(idx->n_sa, 4);
    if (!idx->sa) { fclose(fp); rc = OR_ENOMEM; goto fail; }
    idx->sa[0] = (uint32_t)-1;
    if (fread(idx->sa + 1, 4, idx->n_sa - 1, fp) != idx->n_sa - 1) {
        fclose(fp); rc = OR_EFORMAT; goto fail;
    }
    fclose(fp);
    rc = finish_index(idx);
    if (rc) goto fail;
    free(fn);
    *out = idx;
    return OR_OK;
fail:
    free(fn);
    or_index_free(idx);
    return rc;
}

int or_index_from_arrays(uint32_t primary, const uint32_t L2_1to4[4],
                         const uint32_t *bwt, uint64_t bwt_words,
                         uint32_t sa_intv, const uint32_t *sa_samples,
                         uint64_t n_samples, or_index **out)
{
    *out = NULL;
    or_index *idx = (or_index *)calloc(1, sizeof(or_index));
    if (!idx) return OR_ENOMEM;
    idx->primary = primary;
    idx->L2[0] = 0;
    memcpy(idx->L2 + 1, L2_1to4, 16);
    idx->seq_len = idx->L2[4];
    idx->bwt_words = bwt_words;
    idx->bwt = (uint32_t *)malloc(bwt_words * 4 + 64);
    idx->sa_intv = sa_intv;
    if (sa_intv == 0) { or_index_free(idx); return OR_EINVAL; }
    idx->n_sa = (uint32_t)(((uint64_t)idx->seq_len + sa_intv) / sa_intv);
    idx->sa = (uint32_t *)calloc(idx->n_sa, 4);
    if (!idx->bwt || !idx->sa || n_samples + 1 != idx->n_sa ||
        bwt_words < expected_bwt_words(idx->seq_len)) {
        or_index_free(idx);
        return OR_EINVAL;
    }
    memcpy(idx->bwt, bwt, bwt_words * 4);
    idx->sa[0] = (uint32_t)-1;
    memcpy(idx->sa + 1, sa_samples, n_samples * 4);
    int rc = finish_index(idx);
    if (rc) { or_index_free(idx); return rc; }
    *out = idx;
    return OR_OK;
}

void or_index_free(or_index *idx)
{
    if (!idx) return;
    free(idx->bwt);
    free(idx->sa);
    free(idx);
}

uint32_t or_index_seq_len(const or_index *idx) { return idx->seq_len; }
uint32_t or_index_primary(const or_index *idx) { return idx->primary; }
uint32_t or_index_sa_intv(const or_index *idx) { return idx->sa_intv; }
void or_index_L2(const or_index *idx, uint32_t *L2_out5) { memcpy(L2_out5, idx->L2, 20); }

/* ------------------------------------------------------------------ */
/* occurrence counting: pop_count_full / pop_count_partial (:142-158) and
 * bwt_occ_gpu (:195-216).  Base order inside a word is MSB first (:56). */

static inline uint32_t pc_full(uint32_t w, int c)
{
    uint32_t odd = ((c & 2) ? w : ~w) >> 1;
    uint32_t even = (c & 1) ? w : ~w;
    return (uint32_t)__builtin_popcount(odd & even & 0x55555555u);
}

static inline uint32_t pc_partial(uint32_t w, int c, uint32_t mask_bits)
{
    /* bases after position k in the word are cleared to 00 (= A) and, for
     * c == A, subtracted again */
    w &= ~((1u << (mask_bits << 1)) - 1u);
    uint32_t n = pc_full(w, c);
    return c == 0 ? n - mask_bits : n;
}

/* count of c in the $-removed BWT string positions [0, k] */
static inline uint32_t occ_str(const or_index *idx, uint32_t k, int c)
{
    const uint32_t *blk = idx->bwt + (uint64_t)(k / OCC_INTERVAL) * BLOCK_WORDS;
    uint32_t kw = (k & (OCC_INTERVAL - 1)) >> 4;
    uint32_t n = blk[c];
    for (uint32_t w = 0; w < kw; w++) n += pc_full(blk[4 + w], c);
    return n + pc_partial(blk[4 + kw], c, (~k) & 15u);
}

uint32_t or_occ(const or_index *idx, uint32_t k, int c)
{
    if (k == idx->seq_len) return idx->L2[c + 1] - idx->L2[c];
    if (k == (uint32_t)-1) return 0;
    if (k >= idx->primary) --k;   /* $ is not stored in the BWT string */
    return occ_str(idx, k, c);
}

/* find_occ_gpu (:329-368): occ for both interval ends; returns the number of
 * distinct 64-row blocks it reads (one 32-byte block each). */
static inline int occ_pair(const or_index *idx, uint32_t l, uint32_t u, int c,
                           uint32_t *ol, uint32_t *ou)
{
    if (l == idx->seq_len) { *ol = idx->L2[c + 1] - idx->L2[c]; *ou = or_occ(idx, u, c); return 1; }
    if (u == idx->seq_len) { *ol = or_occ(idx, l, c); *ou = idx->L2[c + 1] - idx->L2[c]; return 1; }
    if (l == (uint32_t)-1) { *ol = 0; *ou = or_occ(idx, u, c); return 1; }
    if (u == (uint32_t)-1) { *ol = or_occ(idx, l, c); *ou = 0; return 1; }
    uint32_t la = l >= idx->primary ? l - 1 : l;
    uint32_t ua = u >= idx->primary ? u - 1 : u;
    *ol = occ_str(idx, la, c);
    *ou = occ_str(idx, ua, c);
    return (la / OCC_INTERVAL == ua / OCC_INTERVAL) ? 1 : 2;
}

void or_occ2(const or_index *idx, uint32_t l, uint32_t u, int c, uint32_t *ol, uint32_t *ou)
{
    occ_pair(idx, l, u, c, ol, ou);
}

/* One backward-search step with base c (:2169-2174, :2321-2326).  A code
 * above 3 leaves the interval unchanged (find_occ_gpu :333). */
static inline int bw_step(const or_index *idx, uint32_t *l, uint32_t *u, int c)
{
    if (c > 3) return 0;
    uint32_t ol, ou;
    int nb = occ_pair(idx, *l - 1, *u, c, &ol, &ou);
    *l = idx->L2[c] + ol + 1;
    *u = idx->L2[c] + ou;
    return nb;
}

/* ------------------------------------------------------------------ */
/* LF / inverse psi (:455-484; bwa form :448-453) and the sampled-SA walk of
 * locate_seeds_gpu (:668-684). */

uint32_t or_lf(const or_index *idx, uint32_t k, int lf_mode)
{
    if (lf_mode == OR_LF_BWA) {
        if (k == idx->primary) return 0;
        uint32_t x = k - (k > idx->primary);
        const uint32_t *blk = idx->bwt + (uint64_t)(x / OCC_INTERVAL) * BLOCK_WORDS;
        int c = (int)((blk[4 + ((x & 63) >> 4)] >> ((~x & 15u) << 1)) & 3u);
        return idx->L2[c] + or_occ(idx, k, c);
    }
    if (k > idx->primary) --k;
    if (k == idx->primary) return 0;          /* also hit by row primary+1 */
    const uint32_t *blk = idx->bwt + (uint64_t)(k / OCC_INTERVAL) * BLOCK_WORDS;
    int c = (int)((blk[4 + ((k & 63) >> 4)] >> ((~k & 15u) << 1)) & 3u);
    if (k == idx->seq_len) return idx->L2[c + 1] - idx->L2[c];
    return idx->L2[c] + occ_str(idx, k, c);
}

uint32_t or_locate(const or_index *idx, uint32_t row, int lf_mode, uint32_t *steps)
{
    uint32_t itr = 0;
    uint64_t cap = (uint64_t)idx->seq_len + 2;
    while (row % idx->sa_intv) {
        itr++;
        row = or_lf(idx, row, lf_mode);
        if (itr > cap) { if (steps) *steps = (uint32_t)-1; return (uint32_t)-1; }
    }
    if (steps) *steps = itr;
    return idx->sa[row / idx->sa_intv] + itr;
}

/* ------------------------------------------------------------------ */
/* k-mer interval table: pre_calc_seed_intervals_gpu (:2648-2675).  Base j of
 * the pattern sits at bits 2j and is processed first. */

typedef struct {
    const or_index *idx;
    int K;
    uint32_t *out;
    uint64_t n;
    int nt, t;
} kmer_job;

static void *kmer_worker(void *arg)
{
    kmer_job *j = (kmer_job *)arg;
    uint64_t per = (j->n + j->nt - 1) / j->nt;
    uint64_t b = per * j->t, e = b + per < j->n ? b + per : j->n;
    for (uint64_t patt = b; patt < e; patt++) {
        uint32_t l = 0, u = j->idx->seq_len;
        for (int i = 0; i < j->K; i++) {
            int ch = (int)((patt >> (i << 1)) & 3u);
            bw_step(j->idx, &l, &u, ch);
            if (l > u) break;
        }
        j->out[2 * patt] = l;
        j->out[2 * patt + 1] = u;
    }
    return NULL;
}

static int default_threads(void)
{
    cpu_set_t cs;
    if (sched_getaffinity(0, sizeof(cs), &cs) == 0) {
        int n = CPU_COUNT(&cs);
        if (n > 0) return n;
    }
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

int or_kmer_table(const or_index *idx, int K, uint32_t *out, int n_threads)
{
    if (K < 1 || K > 15) return OR_EINVAL;
    if (n_threads <= 0) n_threads = default_threads();
    uint64_t n = 1ull << (2 * K);
    kmer_job *jobs = (kmer_job *)calloc((size_t)n_threads, sizeof(kmer_job));
    pthread_t *th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
    if (!jobs || !th) { free(jobs); free(th); return OR_ENOMEM; }
    for (int t = 0; t < n_threads; t++) {
        jobs[t] = (kmer_job){idx, K, out, n, n_threads, t};
        pthread_create(&th[t], NULL, kmer_worker, &jobs[t]);
    }
    for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
    free(jobs);
    free(th);
    return OR_OK;
}

/* ------------------------------------------------------------------ */
/* read encoding: pack_4bit_fow / pack_4bit_rev (:2536-2578).  The code of a
 * character is a nibble of a 32-bit table indexed by its low 3 bits. */

void or_encode(const char *ascii, uint32_t len, uint8_t *fwd, uint8_t *comp)
{
    for (uint32_t i = 0; i < len; i++) {
        uint32_t s = ((uint32_t)(unsigned char)ascii[i] & 7u) << 2;
        if (fwd) fwd[i] = (uint8_t)((0x24031005u >> s) & 15u);
        if (comp) comp[i] = (uint8_t)((0x14002035u >> s) & 15u);
    }
}

/* ------------------------------------------------------------------ */
/* per-candidate search: find_seed_intervals_gpu (:2087-2413) without the
 * warp-shuffle pruning, which only removes records that both filters drop. */

typedef struct {
    int32_t x, y;
    uint32_t l, u;
} cand_rec;

typedef struct {
    uint64_t n_kmer, n_occ_blocks, n_steps, n_lf, n_sa;
} work_ctr;

static inline void kmer_interval(const or_index *idx, const uint32_t *table13,
                                 uint32_t pat, uint32_t *l, uint32_t *u, work_ctr *w)
{
    w->n_kmer++;
    if (table13) {
        *l = table13[2 * (uint64_t)pat];
        *u = table13[2 * (uint64_t)pat + 1];
        return;
    }
    uint32_t a = 0, b = idx->seq_len;
    for (int i = 0; i < K0; i++) {
        bw_step(idx, &a, &b, (int)((pat >> (i << 1)) & 3u));
        if (a > b) break;
    }
    *l = a;
    *u = b;
}

/* Forward strand, candidate end e (:2127-2265). */
static int fwd_candidate(const or_index *idx, const uint32_t *table13, const uint8_t *F,
                         int L, int e, const or_params *p, cand_rec *rec, work_ctr *w,
                         uint32_t *hist, int pruned)
{
    (void)L;
    uint32_t pat = 0;
    int j, i = e;
    for (j = 0; j < K0; j++, i--) {
        int b = F[i];
        if (b > 3) break;
        pat |= (uint32_t)b << (j << 1);
    }
    uint32_t l = 1, u = 0;
    if (j == K0) kmer_interval(idx, table13, pat, &l, &u, w);
    int beg = i;
    if (l <= u) {
        if (pruned) {
            /* containment check at left end e-12 (the 13-mer) */
            uint32_t sz = u - l + 1;
            uint32_t h = hist[e - 12];
            hist[e - 12] = sz;
            if (h == sz) return 0;
        }
        for (; i >= 0; i--) {
            int b = F[i];
            uint32_t nl = l, nu = u;
            if (b <= 3) {
                w->n_occ_blocks += (uint64_t)bw_step(idx, &nl, &nu, b);
                w->n_steps++;
            }
            if (nl > nu) break;
            if (b > 3 && p->n_mode == OR_N_STOP) break;
            l = nl; u = nu; beg = i - 1;
            if (pruned) {
                uint32_t sz = u - l + 1;
                uint32_t h = hist[i];
                hist[i] = sz;
                if (h == sz) return 0;   /* contained in a candidate to the right */
            }
        }
    }
    if (e - beg >= p->k) {
        rec->x = beg + 1;
        rec->y = e + 1;
        rec->l = l;
        rec->u = u;
        return 1;
    }
    return 0;
}

/* Reverse strand (complement codes, not reversed), candidate start s
 * (:2267-2409). */
static int rev_candidate(const or_index *idx, const uint32_t *table13, const uint8_t *C,
                         int L, int s, const or_params *p, cand_rec *rec, work_ctr *w,
                         uint32_t *hist, int pruned)
{
    uint32_t pat = 0;
    int j, i = s;
    for (j = 0; j < K0; j++, i++) {
        int b = C[i];
        if (b > 3) break;
        pat |= (uint32_t)b << (j << 1);
    }
    uint32_t l = 1, u = 0;
    if (j == K0) kmer_interval(idx, table13, pat, &l, &u, w);
    int beg = i;
    if (l > u) return 0;
    if (pruned) {
        uint32_t sz = u - l + 1;
        uint32_t h = hist[s + 12];
        hist[s + 12] = sz;
        if (h == sz) return 0;
    }
    for (; i < L; i++) {
        int b = C[i];
        uint32_t nl = l, nu = u;
        if (b <= 3) {
            w->n_occ_blocks += (uint64_t)bw_step(idx, &nl, &nu, b);
            w->n_steps++;
        }
        if (nl > nu) break;
        if (b > 3 && p->n_mode == OR_N_STOP) break;
        l = nl; u = nu; beg = i + 1;
        if (pruned) {
            uint32_t sz = u - l + 1;
            uint32_t h = hist[i];
            hist[i] = sz;
            if (h == sz) return 0;      /* contained in a candidate to the left */
        }
    }
    if (beg - s >= p->k) {
        rec->x = (int32_t)((uint32_t)s | 0x80000000u);
        rec->y = (int32_t)((uint32_t)beg | 0x80000000u);
        rec->l = l;
        rec->u = u;
        return 1;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* per-read result assembly */

typedef struct {
    or_seed *seeds;
    uint64_t n_seeds, cap_seeds;
    uint32_t *pos;
    uint64_t n_pos, cap_pos;
    work_ctr w;
    int status;
} tbuf;

static int tb_seed(tbuf *t, or_seed s)
{
    if (t->n_seeds == t->cap_seeds) {
        uint64_t nc = t->cap_seeds ? 2 * t->cap_seeds : 1024;
        or_seed *p = (or_seed *)realloc(t->seeds, nc * sizeof(or_seed));
        if (!p) return OR_ENOMEM;
        t->seeds = p;
        t->cap_seeds = nc;
    }
    t->seeds[t->n_seeds++] = s;
    return OR_OK;
}

static int tb_pos(tbuf *t, uint32_t v)
{
    if (t->n_pos == t->cap_pos) {
        uint64_t nc = t->cap_pos ? 2 * t->cap_pos : 4096;
        uint32_t *p = (uint32_t *)realloc(t->pos, nc * 4);
        if (!p) return OR_ENOMEM;
        t->pos = p;
        t->cap_pos = nc;
    }
    t->pos[t->n_pos++] = v;
    return OR_OK;
}

static inline uint32_t isz(const cand_rec *r) { return r->u - r->l + 1u; }

/* Emits rows [l,u] minus the nested interval [xl,xu] (empty when xl > xu)
 * in ascending order, each located by the sampled-SA walk. */
static int emit_rows(const or_index *idx, tbuf *t, const cand_rec *r, uint32_t n,
                     uint32_t xl, uint32_t xu, int lf_mode)
{
    uint32_t done = 0;
    for (uint32_t row = r->l; done < n; row++) {
        if (xl <= xu && row >= xl && row <= xu) continue;
        uint32_t steps;
        uint32_t pos = or_locate(idx, row, lf_mode, &steps);
        if (steps == (uint32_t)-1) return OR_EWALK;
        t->w.n_lf += steps;
        t->w.n_sa++;
        if (tb_pos(t, pos)) return OR_ENOMEM;
        done++;
    }
    return OR_OK;
}

/* Filters, orders and locates one read's records.
 *   SMEM: filter_seed_intervals_gpu (:991-1019), stable segmented sort by
 *         begin (:1233), count_seed_intervals_gpu (:865-880),
 *         seeds_to_threads + locate_seeds_gpu (:555-573, :668-684).
 *   MEM:  filter_seed_intervals_gpu_mem (:1103-1139), count (:927-989),
 *         seeds_to_threads_mem (:624-667), locate, stable segmented sort of
 *         positions by begin (:3566-3571). */
static int finish_read(const or_index *idx, const or_params *p, cand_rec *fw, int nf,
                       cand_rec *rv, int nr, tbuf *t, uint32_t *n_seeds_out)
{
    uint32_t ns = 0;
    /* filtered copies: dropped records become (1,0) */
    if (p->smem) {
        for (int o = 0; o + 1 < nf; o++)
            if (fw[o + 1].x == fw[o].x) { fw[o].l = 1; fw[o].u = 0; }
        for (int o = nr - 1; o >= 1; o--)
            if (rv[o].y == rv[o - 1].y) { rv[o].l = 1; rv[o].u = 0; }
    } else {
        /* decisions use the unfiltered neighbour, as the reference reads the
         * compacted input while writing the filtered output */
        uint32_t *keepf = (uint32_t *)malloc(sizeof(uint32_t) * (nf + 1));
        uint32_t *keepr = (uint32_t *)malloc(sizeof(uint32_t) * (nr + 1));
        if (!keepf || !keepr) { free(keepf); free(keepr); return OR_ENOMEM; }
        for (int o = 0; o < nf; o++)
            keepf[o] = !(o + 1 < nf && fw[o + 1].x == fw[o].x && isz(&fw[o + 1]) == isz(&fw[o]));
        for (int o = 0; o < nr; o++)
            keepr[o] = !(o > 0 && rv[o].y == rv[o - 1].y && isz(&rv[o]) == isz(&rv[o - 1]));
        for (int o = 0; o < nf; o++) if (!keepf[o]) { fw[o].l = 1; fw[o].u = 0; }
        for (int o = 0; o < nr; o++) if (!keepr[o]) { rv[o].l = 1; rv[o].u = 0; }
        free(keepf);
        free(keepr);
    }
    /* merge by begin; ties keep the forward record first (stable sort of
     * [fwd..., rev...]) */
    int a = 0, b = 0;
    while (a < nf || b < nr) {
        int take_f;
        if (a >= nf) take_f = 0;
        else if (b >= nr) take_f = 1;
        else take_f = (uint32_t)(fw[a].x & 0x7fffffff) <= (uint32_t)(rv[b].x & 0x7fffffff);
        cand_rec *r = take_f ? &fw[a] : &rv[b];
        uint32_t n = isz(r);
        uint32_t xl = 1, xu = 0;
        if (!p->smem && n > 0) {
            /* next valid record of the same run, toward the longer match */
            if (take_f) {
                for (int q = a + 1; q < nf && fw[q].x == r->x; q++)
                    if (isz(&fw[q]) > 0) { xl = fw[q].l; xu = fw[q].u; n -= isz(&fw[q]); break; }
            } else {
                for (int q = b - 1; q >= 0 && rv[q].y == r->y; q--)
                    if (isz(&rv[q]) > 0) { xl = rv[q].l; xu = rv[q].u; n -= isz(&rv[q]); break; }
            }
        }
        if (n > 0) {
            or_seed s = {r->x, r->y, r->l, r->u, n};
            if (tb_seed(t, s)) return OR_ENOMEM;
            int rc = emit_rows(idx, t, r, n, xl, xu, p->lf_mode);
            if (rc) return rc;
            ns++;
        }
        if (take_f) a++; else b++;
    }
    *n_seeds_out = ns;
    return OR_OK;
}

/* MEM mode, mem_next = 1: seeds_to_threads_mem (:635-650) scans for a
 * record's exclusion interval through the batch's compacted records, past
 * the read's end, while count_seed_intervals_gpu_mem (:927-989) counts
 * within the read.  The scan leaves the read only from its last forward
 * record when the read has no reverse record (the next array record is the
 * next read's first; it matters when it is forward with the same begin) and
 * from its first reverse record when the read has no forward record (the
 * previous read's last record, reverse with the same end).  That record
 * starts (ends) a run whose last (first) record is kept, and a dropped
 * record has the interval of the one it was dropped for, so the first
 * non-empty interval the scan meets is that of the other read's first
 * forward (last reverse) output seed.  The seed keeps its count and its
 * rows become the first n_pos rows from l outside that interval (the
 * reference's emission loop, :655-662).  Runs after every read is done. */
static int mem_next_pass(const or_index *idx, const or_params *p, or_batch *bt)
{
    for (uint32_t r = 0; r < bt->n_reads; r++) {
        uint64_t s0 = bt->read_seed_off[r], s1 = bt->read_seed_off[r + 1];
        if (s0 == s1) continue;
        uint64_t last_f = s1, first_r = s1;
        for (uint64_t s = s0; s < s1; s++) {
            if ((uint32_t)bt->seeds[s].y >> 31) { if (first_r == s1) first_r = s; }
            else last_f = s;
        }
        uint64_t target = s1;
        const or_seed *J = NULL;
        if (last_f < s1 && first_r == s1) {
            uint32_t q = r + 1;
            while (q < bt->n_reads && bt->read_seed_off[q + 1] == bt->read_seed_off[q]) q++;
            if (q < bt->n_reads)
                for (uint64_t s = bt->read_seed_off[q]; s < bt->read_seed_off[q + 1]; s++) {
                    if ((uint32_t)bt->seeds[s].y >> 31) continue;
                    if (bt->seeds[s].x == bt->seeds[last_f].x) { J = &bt->seeds[s]; target = last_f; }
                    break;
                }
        } else if (first_r < s1 && last_f == s1 && r > 0) {
            uint32_t q = r - 1;
            while (q > 0 && bt->read_seed_off[q + 1] == bt->read_seed_off[q]) q--;
            for (uint64_t s = bt->read_seed_off[q + 1]; s-- > bt->read_seed_off[q];) {
                if (!((uint32_t)bt->seeds[s].y >> 31)) continue;
                if (bt->seeds[s].y == bt->seeds[first_r].y) { J = &bt->seeds[s]; target = first_r; }
                break;
            }
        }
        if (!J) continue;
        uint64_t pos = bt->read_pos_off[r];
        for (uint64_t s = s0; s < target; s++) pos += bt->seeds[s].n_pos;
        const or_seed *S = &bt->seeds[target];
        uint32_t done = 0;
        for (uint32_t row = S->l; done < S->n_pos; row++) {
            if (row >= J->l && row <= J->u) continue;
            uint32_t steps;
            uint32_t v = or_locate(idx, row, p->lf_mode, &steps);
            if (steps == (uint32_t)-1) return OR_EWALK;
            bt->pos[pos + done++] = v;
        }
    }
    return OR_OK;
}

/* ------------------------------------------------------------------ */
/* batch driver */

typedef struct {
    const or_index *idx;
    const uint32_t *table13;
    const char *seqs;
    const uint64_t *offsets;
    const uint32_t *lengths;
    uint32_t n_reads;
    const or_params *p;
    int pruned;
    volatile uint32_t next;
    uint32_t *read_thread;     /* which thread produced read r */
    uint64_t *read_seed_start, *read_pos_start;
    uint32_t *read_n_seeds;
    uint64_t *read_n_pos;
    uint32_t *read_n_fwd;
} batch_ctx;

typedef struct {
    batch_ctx *ctx;
    int tid;
    tbuf tb;
} worker_arg;

static void *seed_worker(void *arg)
{
    worker_arg *wa = (worker_arg *)arg;
    batch_ctx *c = wa->ctx;
    tbuf *t = &wa->tb;
    uint8_t *F = NULL, *C = NULL;
    uint32_t *hist = NULL;
    cand_rec *fw = NULL, *rv = NULL;
    uint32_t cap = 0;
    for (;;) {
        uint32_t r0 = __atomic_fetch_add(&c->next, 16u, __ATOMIC_RELAXED);
        if (r0 >= c->n_reads || t->status) break;
        uint32_t r1 = r0 + 16 < c->n_reads ? r0 + 16 : c->n_reads;
        for (uint32_t r = r0; r < r1; r++) {
            uint32_t L = c->lengths[r];
            if (L + 1 > cap) {
                cap = L + 1;
                F = (uint8_t *)realloc(F, cap);
                C = (uint8_t *)realloc(C, cap);
                hist = (uint32_t *)realloc(hist, sizeof(uint32_t) * cap);
                fw = (cand_rec *)realloc(fw, sizeof(cand_rec) * cap);
                rv = (cand_rec *)realloc(rv, sizeof(cand_rec) * cap);
                if (!F || !C || !hist || !fw || !rv) { t->status = OR_ENOMEM; break; }
            }
            c->read_thread[r] = (uint32_t)wa->tid;
            c->read_seed_start[r] = t->n_seeds;
            c->read_pos_start[r] = t->n_pos;
            uint64_t p0 = t->n_pos;
            uint32_t ns = 0;
            int k = c->p->k;
            if ((int)L >= k) {
                or_encode(c->seqs + c->offsets[r], L, F, C);
                int nf = 0, nr = 0;
                /* forward candidates are produced right to left; records are
                 * kept in ascending end order (:2261) */
                if (c->pruned) memset(hist, 0, sizeof(uint32_t) * L);
                for (int e = (int)L - 1; e >= k - 1; e--) {
                    cand_rec rec;
                    if (fwd_candidate(c->idx, c->table13, F, (int)L, e, c->p, &rec, &t->w,
                                      hist, c->pruned))
                        fw[nf++] = rec;
                }
                for (int q = 0; q < nf / 2; q++) {
                    cand_rec tmp = fw[q]; fw[q] = fw[nf - 1 - q]; fw[nf - 1 - q] = tmp;
                }
                if (c->pruned) memset(hist, 0, sizeof(uint32_t) * L);
                for (int s = 0; s <= (int)L - k; s++) {
                    cand_rec rec;
                    if (rev_candidate(c->idx, c->table13, C, (int)L, s, c->p, &rec, &t->w,
                                      hist, c->pruned))
                        rv[nr++] = rec;
                }
                c->read_n_fwd[r] = (uint32_t)nf;
                int rc = finish_read(c->idx, c->p, fw, nf, rv, nr, t, &ns);
                if (rc) { t->status = rc; break; }
            }
            c->read_n_seeds[r] = ns;
            c->read_n_pos[r] = t->n_pos - p0;
        }
    }
    free(F); free(C); free(hist); free(fw); free(rv);
    return NULL;
}

int or_seed_batch(const or_index *idx, const uint32_t *table13,
                  const char *seqs, const uint64_t *offsets,
                  const uint32_t *lengths, uint32_t n_reads,
                  const or_params *p, int pruned, int n_threads,
                  or_batch **out)
{
    *out = NULL;
    if (p->k < K0) return OR_EINVAL;   /* k < 13 reads outside the read */
    if (n_threads <= 0) n_threads = default_threads();
    if ((uint32_t)n_threads > n_reads / 16 + 1) n_threads = (int)(n_reads / 16 + 1);
    batch_ctx c;
    memset(&c, 0, sizeof(c));
    c.idx = idx; c.table13 = table13; c.seqs = seqs; c.offsets = offsets;
    c.lengths = lengths; c.n_reads = n_reads; c.p = p; c.pruned = pruned;
    c.read_thread = (uint32_t *)calloc(n_reads + 1, 4);
    c.read_seed_start = (uint64_t *)calloc(n_reads + 1, 8);
    c.read_pos_start = (uint64_t *)calloc(n_reads + 1, 8);
    c.read_n_seeds = (uint32_t *)calloc(n_reads + 1, 4);
    c.read_n_pos = (uint64_t *)calloc(n_reads + 1, 8);
    c.read_n_fwd = (uint32_t *)calloc(n_reads + 1, 4);
    worker_arg *wa = (worker_arg *)calloc((size_t)n_threads, sizeof(worker_arg));
    pthread_t *th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
    or_batch *bt = (or_batch *)calloc(1, sizeof(or_batch));
    int rc = OR_OK;
    if (!c.read_thread || !c.read_seed_start || !c.read_pos_start || !c.read_n_seeds ||
        !c.read_n_pos || !wa || !th || !bt) { rc = OR_ENOMEM; goto done; }
    for (int t = 0; t < n_threads; t++) {
        wa[t].ctx = &c;
        wa[t].tid = t;
        pthread_create(&th[t], NULL, seed_worker, &wa[t]);
    }
    for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
    for (int t = 0; t < n_threads; t++) if (wa[t].tb.status) rc = wa[t].tb.status;
    if (rc) goto done;

    /* gather per-thread buffers in read order */
    bt->n_reads = n_reads;
    bt->read_n_seeds = c.read_n_seeds; c.read_n_seeds = NULL;
    bt->read_n_fwd = c.read_n_fwd; c.read_n_fwd = NULL;
    bt->read_seed_off = (uint64_t *)calloc(n_reads + 1, 8);
    bt->read_pos_off = (uint64_t *)calloc(n_reads + 1, 8);
    if (!bt->read_seed_off || !bt->read_pos_off) { rc = OR_ENOMEM; goto done; }
    for (uint32_t r = 0; r < n_reads; r++) {
        bt->read_seed_off[r + 1] = bt->read_seed_off[r] + bt->read_n_seeds[r];
        bt->read_pos_off[r + 1] = bt->read_pos_off[r] + c.read_n_pos[r];
    }
    bt->n_seeds = bt->read_seed_off[n_reads];
    bt->n_pos = bt->read_pos_off[n_reads];
    bt->seeds = (or_seed *)malloc(sizeof(or_seed) * (bt->n_seeds + 1));
    bt->pos = (uint32_t *)malloc(4 * (bt->n_pos + 1));
    if (!bt->seeds || !bt->pos) { rc = OR_ENOMEM; goto done; }
    for (uint32_t r = 0; r < n_reads; r++) {
        tbuf *t = &wa[c.read_thread[r]].tb;
        memcpy(bt->seeds + bt->read_seed_off[r], t->seeds + c.read_seed_start[r],
               sizeof(or_seed) * bt->read_n_seeds[r]);
        memcpy(bt->pos + bt->read_pos_off[r], t->pos + c.read_pos_start[r],
               4 * c.read_n_pos[r]);
    }
    if (!p->smem && p->mem_next) {
        rc = mem_next_pass(idx, p, bt);
        if (rc) goto done;
    }
    for (int t = 0; t < n_threads; t++) {
        bt->n_kmer += wa[t].tb.w.n_kmer;
        bt->n_occ_blocks += wa[t].tb.w.n_occ_blocks;
        bt->n_steps += wa[t].tb.w.n_steps;
        bt->n_lf += wa[t].tb.w.n_lf;
        bt->n_sa += wa[t].tb.w.n_sa;
    }
done:
    if (wa) for (int t = 0; t < n_threads; t++) { free(wa[t].tb.seeds); free(wa[t].tb.pos); }
    free(wa); free(th);
    free(c.read_thread); free(c.read_seed_start); free(c.read_pos_start);
    free(c.read_n_seeds); free(c.read_n_pos); free(c.read_n_fwd);
    if (rc) { or_batch_free(bt); return rc; }
    *out = bt;
    return OR_OK;
}

void or_batch_free(or_batch *b)
{
    if (!b) return;
    free(b->read_n_seeds); free(b->read_seed_off); free(b->read_pos_off); free(b->read_n_fwd);
    free(b->seeds); free(b->pos);
    free(b);
}

/* ------------------------------------------------------------------ */
/* text records (:3625-3647) */

int or_batch_write_text(const or_batch *b, const char *path, uint32_t first_read_no,
                        int smem, int append)
{
    FILE *fp = fopen(path, append ? "ab" : "wb");
    if (!fp) return OR_EIO;
    static const char sign[2] = {'+', '-'};
    for (uint32_t r = 0; r < b->n_reads; r++) {
        fprintf(fp, "/*===================================%s seeds in read no. %u "
                    "(Read[begin, End] -> starting position(s) on the reference)"
                    "===================================*/\n",
                smem ? "SMEM" : "MEM", first_read_no + r);
        int32_t pb = -1, pe = -1;
        uint64_t s0 = b->read_seed_off[r], s1 = b->read_seed_off[r + 1];
        const uint32_t *pos = b->pos + b->read_pos_off[r];
        for (uint64_t s = s0; s < s1; s++) {
            const or_seed *sd = &b->seeds[s];
            for (uint32_t q = 0; q < sd->n_pos; q++, pos++) {
                char sg = sign[((uint32_t)sd->y) >> 31];
                if (pb == sd->x && pe == sd->y)
                    fprintf(fp, ", %c%u", sg, *pos);
                else
                    fprintf(fp, "\nRead[%d, %d] -> %c%u", (int)((uint32_t)sd->x & 0x7fffffffu),
                            (int)((uint32_t)sd->y & 0x7fffffffu), sg, *pos);
                pb = sd->x;
                pe = sd->y;
            }
        }
        fputc('\n', fp);
    }
    fclose(fp);
    return OR_OK;
}
