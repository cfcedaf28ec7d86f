/*
 * oracle.h -- CPU restatement of GPUseed's seeding path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (gpuseed_gb300/, the
 * seed_gen CLI, the C-ABI library) links, loads or calls this code.  Only
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it,
 * and only as the checker or as the timed CPU baseline.
 *
 * Every function restates one piece of the reference (nahmedraja/GPUseed,
 * single file seed_gen.cu) and cites the lines it follows.  The reference has
 * no tests, fixtures or golden vectors; the restatement is pinned by
 *   (1) a brute-force substring matcher (tests/bruteforce.py, tests/golden/),
 *   (2) a CPU build of the reference's own kernel bodies
 *       (oracle/ref_emul/, built into oracle/_ref/ from the reference tree
 *       when it is present), compared on seeded inputs.
 *
 * Semantics switches for the reference's undefined behaviour:
 *   n_mode  OR_N_WILDCARD (default): a non-ACGT base after the first 13
 *           leaves the interval unchanged and the match continues
 *           (seed_gen.cu:2125/2246/2387 read an uninitialised `base`, which a
 *           compiler folds to "not > 3"; find_occ_gpu at :333 returns the
 *           interval unchanged for c > 3).
 *           OR_N_STOP: the extension stops at such a base (bwa behaviour).
 *   lf_mode OR_LF_GPUSEED (default): LF(primary+1) == 0 as bwt_inv_psi_gpu
 *           (seed_gen.cu:455-458) computes it.
 *           OR_LF_BWA: LF as bwa computes it (seed_gen.cu:448-453).
 */
#ifndef GPUSEED_ORACLE_H
#define GPUSEED_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_N_WILDCARD = 0, OR_N_STOP = 1 };
enum { OR_LF_GPUSEED = 0, OR_LF_BWA = 1 };

/* Index in the reference's in-memory form (seed_gen.cu:37-46): bwtint_t is
 * uint32_t (:22), 64-row occurrence blocks of 4 counts + 4 BWT words (:29,
 * :52-58), L2[0..4], sampled SA with sa[0] == (uint32_t)-1 (:2711). */
typedef struct {
    uint32_t primary;
    uint32_t L2[5];
    uint32_t seq_len;
    uint64_t bwt_words;   /* words in bwt[] */
    uint32_t *bwt;
    uint32_t sa_intv;
    uint32_t n_sa;
    uint32_t *sa;
} or_index;

typedef struct {
    int32_t k;        /* -k: minimum seed length (seed_gen.cu:2820) */
    int32_t smem;     /* -s: SMEM mode; 0 = MEM mode (seed_gen.cu:2831) */
    int32_t n_mode;   /* OR_N_WILDCARD / OR_N_STOP */
    int32_t lf_mode;  /* OR_LF_GPUSEED / OR_LF_BWA */
    int32_t mem_next; /* 0: a MEM record's exclusion interval from its own read;
                         1: also across reads, as seeds_to_threads_mem's scan
                         (seed_gen.cu:635-650) finds it */
} or_params;

/* One output seed: the reference's int2 read position (x = begin, y = end
 * exclusive, bit 31 of both set on the '-' strand; seed_gen.cu:2262, :2402),
 * its SA interval and the number of positions it emits. */
typedef struct {
    int32_t x, y;
    uint32_t l, u;
    uint32_t n_pos;
} or_seed;

typedef struct {
    uint32_t n_reads;
    uint32_t *read_n_seeds;    /* per read */
    uint64_t *read_seed_off;   /* per read, into seeds[] (n_reads+1) */
    uint64_t *read_pos_off;    /* per read, into pos[] (n_reads+1) */
    uint64_t n_seeds, n_pos;
    or_seed *seeds;
    uint32_t *pos;
    /* algorithmic work counters (32-byte units), summed over reads */
    uint64_t n_kmer, n_occ_blocks, n_lf, n_sa, n_steps;
    int32_t status;            /* 0 or negative error */
    uint32_t *read_n_fwd;      /* per read: forward records before the filters
                                  (full walk only; the reference's MEM filter
                                  leaves the single record of a read with
                                  exactly one unwritten, seed_gen.cu:1110) */
} or_batch;

/* ---- index ---------------------------------------------------------- */
int  or_index_load(const char *prefix, or_index **out);
int  or_index_from_arrays(uint32_t primary, const uint32_t L2_1to4[4],
                          const uint32_t *bwt, uint64_t bwt_words,
                          uint32_t sa_intv, const uint32_t *sa_samples,
                          uint64_t n_samples, or_index **out);
void or_index_free(or_index *idx);
uint32_t or_index_seq_len(const or_index *idx);
uint32_t or_index_primary(const or_index *idx);
uint32_t or_index_sa_intv(const or_index *idx);
void or_index_L2(const or_index *idx, uint32_t *L2_out5);

/* ---- FM primitives -------------------------------------------------- */
uint32_t or_occ(const or_index *idx, uint32_t k, int c);
void     or_occ2(const or_index *idx, uint32_t l, uint32_t u, int c,
                 uint32_t *ol, uint32_t *ou);
uint32_t or_lf(const or_index *idx, uint32_t row, int lf_mode);
/* SA value of `row` by the sampled-SA walk; *steps gets the walk length. */
uint32_t or_locate(const or_index *idx, uint32_t row, int lf_mode, uint32_t *steps);

/* ---- k-mer interval table (seed_gen.cu:2648-2675) ------------------- */
/* out holds 2*4^K uint32: (l,u) per pattern. n_threads <= 0: all cores. */
int or_kmer_table(const or_index *idx, int K, uint32_t *out, int n_threads);

/* ---- read encoding (seed_gen.cu:2536-2578) -------------------------- */
void or_encode(const char *ascii, uint32_t len, uint8_t *fwd, uint8_t *comp);

/* ---- seeding --------------------------------------------------------- */
/* Seeds a batch of reads given as concatenated ASCII with per-read offsets
 * and lengths.  pruned == 0: every candidate extended to its end (the
 * checker).  pruned == 1: containment-stopped walk (the CPU baseline; same
 * output).  n_threads <= 0: all cores. */
int or_seed_batch(const or_index *idx, const uint32_t *table13,
                  const char *seqs, const uint64_t *offsets,
                  const uint32_t *lengths, uint32_t n_reads,
                  const or_params *p, int pruned, int n_threads,
                  or_batch **out);
void or_batch_free(or_batch *b);

/* Text records exactly as seed_gen -o prints them (seed_gen.cu:3625-3647).
 * first_read_no is the 1-based number of the batch's first read. */
int or_batch_write_text(const or_batch *b, const char *path, uint32_t first_read_no,
                        int smem, int append);

/* ---- index construction (test fixtures) ----------------------------- */
/* Builds the .bwt/.sa pair of a forward-strand text of codes 0..3 with the
 * layout the reference reads (seed_gen.cu:2685-2736, :52-58). */
int or_build_index(const uint8_t *codes, uint64_t n, uint32_t sa_intv,
                   const char *prefix);
/* Suffix array of codes[0..n) plus the sentinel: sa_out has n+1 entries,
 * sa_out[0] == n. */
int or_suffix_array(const uint8_t *codes, uint64_t n, uint32_t *sa_out);

#ifdef __cplusplus
}
#endif
#endif
