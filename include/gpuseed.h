/*
 * gpuseed.h -- C-ABI of the GB300 seeding library (libgpuseed.so).
 *
 * The reference (nahmedraja/GPUseed) has no library interface: its boundary is
 * the seed_gen process, the .bwt/.sa index files and the text records on
 * stdout (seed_gen.cu:2817-3815).  These entry points are what a caller of
 * that path binds instead; each comment names the reference code it replaces.
 * Plain pointers and sizes only.  Every call returns 0 or a negative GS_E*
 * code and never exits; gs_last_error() describes the last failure of the
 * calling thread.
 *
 * Threading: a gs_index may be shared by threads; it changes only through
 * gs_index_set_kmer_len / _set_text / _set_l2_window, which must not overlap
 * a pass on any of its contexts (a context's captured pass is captured
 * again after such a change).  A gs_ctx (stream + workspace + last result)
 * belongs to one host thread at a time.  A call makes its index's device
 * current while it runs and gives the calling thread its previous current
 * device back before it returns.
 */
#ifndef GPUSEED_H
#define GPUSEED_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GS_OK 0
#define GS_EINVAL -1     /* bad argument */
#define GS_EIO -2        /* file cannot be opened or read */
#define GS_EFORMAT -3    /* index file truncated or inconsistent */
#define GS_ENOMEM -4     /* device or host allocation failed / admission refused */
#define GS_ECUDA -5      /* CUDA runtime error */
#define GS_EWALK -6      /* sampled-SA walk exceeded its step limit (corrupt index) */
#define GS_EOVERFLOW -7  /* output larger than the capacity given */
#define GS_ETIMEOUT -8   /* a bounded wait ran out */
#define GS_ESTATE -9     /* call not valid in the object's current state */

/* Semantics switches (defaults first: the reference's behaviour). */
#define GS_N_WILDCARD 0  /* non-ACGT base after the 13-mer: interval unchanged, as the
                            reference's unassigned `base` test and find_occ_gpu's early
                            return make it (seed_gen.cu:2125, :2246, :333) */
#define GS_N_STOP 1      /* non-ACGT base stops the extension (bwa) */
#define GS_LF_GPUSEED 0  /* LF(primary+1) = 0 as seed_gen.cu:455-458 */
#define GS_LF_BWA 1      /* LF as bwa */

/* MEM mode: where a kept record's exclusion interval (the nested interval of
 * its neighbour toward the longer match) may come from. */
#define GS_MEM_NEXT_READ 0     /* the same read only: a read's seeds do not depend on the
                                  other reads of the batch (default; serving needs it) */
#define GS_MEM_NEXT_GPUSEED 1  /* as seeds_to_threads_mem (seed_gen.cu:635-650), whose scan
                                  for the neighbour does not stop at the read's end: a
                                  read's last forward seed, when the read has no reverse
                                  seed, takes the first forward seed of the next read with
                                  seeds if it has the same begin (and a read's first
                                  reverse seed, when the read has no forward seed, the
                                  last reverse seed of the previous one if it has the
                                  same end); it keeps its count and emits the first
                                  n_pos rows from l outside that interval */

#define GS_KERNEL_BATCHED 0  /* candidates started a warp per work item, then walked one per
                                lane, each with its neighbour's interval (default) */
#define GS_KERNEL_PLAIN 1    /* one read per thread */
#define GS_KERNEL_LOCKSTEP 2 /* a warp steps 31 candidates in lockstep, comparing neighbours by
                                shuffles, and hands its last ones to a tail pass */

typedef struct gs_index gs_index;
typedef struct gs_ctx gs_ctx;

/* seed_gen's -k / -s switches (seed_gen.cu:2820-2839) plus the quirk modes. */
typedef struct {
    int32_t k;          /* minimum seed length, >= 13 (default 20) */
    int32_t smem;       /* 1: SMEM mode (-s); 0: MEM mode */
    int32_t n_mode;     /* GS_N_WILDCARD | GS_N_STOP */
    int32_t lf_mode;    /* GS_LF_GPUSEED | GS_LF_BWA */
    int32_t kernel;     /* GS_KERNEL_BATCHED | GS_KERNEL_PLAIN | GS_KERNEL_LOCKSTEP */
    int32_t queue_chunk;    /* work items a warp takes per queue grab (0 = auto) */
    int32_t ctas_per_sm;    /* persistent CTAs per SM (0 = auto) */
    int32_t count_work;     /* 1: count algorithmic work (plain kernel walk + locate) */
    int32_t handoff_lanes;  /* lockstep: a warp hands its last extending candidates to a
                               tail pass once at most this many remain (0 = auto, <0 = never) */
    int32_t handoff_steps;  /* ... but not before this many lockstep steps (0 = auto) */
    int32_t graph;          /* gs_seed_device: 1 = capture the pass into a CUDA graph on the
                               first call and replay it while the inputs (pointers, n_reads,
                               params) repeat; outputs that outgrow the captured capacities
                               fall back to a sized pass and a new capture */
    int32_t walker_slots;   /* batched: walker buffer entries per 16 work items of 31
                               candidates, a work item of 30 read windows (both strands)
                               counting as two (0 = auto, 256; <0 = none: walks that
                               outlast their start run in a later pass, unpruned) */
    int32_t max_occ;        /* > 0: drop output seeds whose interval has more rows than this
                               (bwa's -c; applied after the filters, the other seeds are
                               unchanged); 0 = off, the reference's output */
    int32_t mem_next;       /* GS_MEM_NEXT_READ | GS_MEM_NEXT_GPUSEED (MEM mode only; a
                               batch then runs as one pass, and servers refuse it) */
} gs_params;

/* One output seed, in output order.  x/y are the reference's int2 read
 * position (begin, exclusive end; bit 31 of both set on the '-' strand,
 * seed_gen.cu:2262, :2402).  Its positions are the first n_pos rows from l
 * that lie outside [xl,xu] (empty when xl > xu): rows [l,u] minus the nested
 * interval [xl,xu] in MEM mode; with GS_MEM_NEXT_GPUSEED, [xl,xu] may be
 * another read's interval that overlaps [l,u] without being nested, and the
 * rows then run past u. */
typedef struct {
    int32_t x, y;
    uint32_t l, u;
    uint32_t xl, xu;
    uint32_t n_pos;
    uint32_t pad;
} gs_seed_rec;

typedef struct {
    uint32_t n_reads;
    uint64_t n_seeds;
    uint64_t n_pos;
    const uint64_t *read_seed_off;  /* n_reads + 1 */
    const uint64_t *read_pos_off;   /* n_reads + 1 */
    const gs_seed_rec *seeds;           /* n_seeds */
    const uint32_t *pos;            /* n_pos reference positions, output order */
} gs_result_view;

typedef struct {
    uint32_t seq_len, primary, sa_intv, n_sa;
    uint32_t L2[5];
    int32_t device;
    uint64_t device_bytes;          /* HBM held by the index */
    int32_t kmer_len;               /* start-table length in use (13..16) */
    int32_t text_min;               /* text structures: > 0 the min_steps of
                                       gs_index_set_text, -1 built but text mode off,
                                       0 not built */
} gs_index_info;

/* ---- index -------------------------------------------------------------
 * Replaces bwt_restore_bwt / bwt_restore_sa + the H2D copies and the 13-mer
 * table precalculation of seed_gen.cu:2685-2736, :2841-2895. */
int gs_index_load(const char *prefix, int device, gs_index **out);
/* Same from memory: .bwt words after the 5-word header and the .sa samples
 * after its 7-word header. */
int gs_index_from_host(uint32_t primary, const uint32_t L2_1to4[4], const uint32_t *bwt,
                       uint64_t bwt_words, uint32_t sa_intv, const uint32_t *sa_samples,
                       uint64_t n_samples, int device, gs_index **out);
void gs_index_free(gs_index *idx);
int gs_index_get_info(const gs_index *idx, gs_index_info *out);
/* Copies the device 13-mer table (2*4^13 uint32: l,u per pattern) or a
 * range of it to host memory (pre_calc_seed_intervals_gpu, seed_gen.cu:2648). */
int gs_index_kmer_table(const gs_index *idx, uint64_t first, uint64_t count, uint32_t *out);
/* Index construction, replacing build_index.sh (bwa index -b sa -r R and
 * bwa index -b bwt, build_index.sh:36-75): suffix array of the forward-strand
 * text on the GPU, BWT, 64-row occurrence blocks and the row-sampled SA, in
 * the file layout seed_gen.cu:2685-2736 reads.  codes: n bytes in 0..3.
 * Writes <prefix>.bwt and <prefix>.sa when prefix is not NULL; loads the
 * index on `device` into *out when out is not NULL. */
int gs_index_build(const uint8_t *codes, uint64_t n, uint32_t sa_intv, int device,
                   const char *prefix, gs_index **out);
/* Length of the k-mer start table (13..16).  Loading picks 16 above 2^30
 * bases, 15 above 2^28, 14 above 2^26, else 13 (16 * 4^len bytes of HBM:
 * each len-mer's entry and its reverse complement's, so that one lookup
 * starts both strands' candidates of a read window; a lower length is taken
 * when the memory is not there).  A candidate starts from the interval of
 * its first len bases instead of 13 + len-13 steps: the SA interval of a
 * string does not depend on how it is found, so results do not change;
 * seeding uses it only when k > len.  Call while no pass runs on a context
 * of this index. */
int gs_index_set_kmer_len(gs_index *idx, int kmer_len);
/* Text structures in HBM, built from the .bwt and .sa by one pass of LF
 * chains: 4 * seq_len bytes of full suffix array, seq_len / 4 of packed
 * text, 2 * seq_len of inverse-SA samples every 2 positions (19.4 GB and
 * 0.3-0.5 s at 3.1 Gbp).  Loading does not build them: on config-3 reads
 * they save ~1.6 ms per million reads, so they pay for their build after a
 * few hundred million reads.  min_steps 4 is the measured best.  With them,
 * locate reads each
 * position from the full suffix array instead of walking to a sampled row,
 * and a walker whose interval has been one row, with its containment test
 * over, for min_steps steps (so that the row is the read's own locus, not a
 * chance hit) compares its read with the text, 16 bases a step, in a pass
 * of its own; it takes the row where the match ends from the inverse-SA
 * samples.  Seeds and positions do not change.  min_steps > 0: build if
 * needed and use both; < 0: build if needed, locate only; 0: free them.
 * Call while no pass runs on a context of this index. */
int gs_index_set_text(gs_index *idx, int min_steps);
/* Copies entries [first, first+count) of a text structure to host memory:
 * which 0 = full suffix array (seq_len+1 rows), 1 = packed text words
 * (ceil(seq_len/16)), 2 = inverse-SA samples (seq_len/2 + 1). */
int gs_index_text_table(const gs_index *idx, int which, uint64_t first, uint64_t count,
                        uint32_t *out);
/* Keeps the occurrence table in L2 under an access-policy window on the
 * streams of contexts created afterwards (fraction of the set-aside; 0, the
 * default, disables it and releases the set-aside).  Measured slower on the
 * search's random accesses (70.9 -> 94.4 ms, 4M reads on 3.1 Gbp): off
 * unless asked for. */
int gs_index_set_l2_window(gs_index *idx, float hit_ratio);

/* ---- seeding context ---------------------------------------------------
 * One pass over a batch of reads replaces seed_gen's per-batch loop body
 * (seed_gen.cu:3029-3620): pack, search, compaction, filters, sort, locate. */
int gs_ctx_create(gs_index *idx, void *cuda_stream, gs_ctx **out);
void gs_ctx_free(gs_ctx *ctx);
/* Reads in host memory (ASCII, one record per read, offsets in bytes):
 * copies them in, seeds, and copies the result back to host memory owned by
 * the context (valid until the next call on it).  A batch of 2^22 reads or
 * more whose reads lie in order in `seqs` runs as up to 16 chunks: each
 * chunk's reads are copied in while the chunks before it run, and its
 * results are copied out while the next one runs.  The host result is the
 * same; the device then holds only the last chunk's, so gs_result_device
 * and gs_result_text_device return GS_ESTATE and gs_result_write_text
 * formats on the host. */
int gs_seed(gs_ctx *ctx, const char *seqs, const uint64_t *offsets, const uint32_t *lengths,
            uint32_t n_reads, const gs_params *p);
/* Reads already in device memory; fetch_to_host = 0 leaves the result on the
 * device (gs_result_device). */
int gs_seed_device(gs_ctx *ctx, const char *d_seqs, const uint64_t *d_offsets,
                   const uint32_t *d_lengths, uint32_t n_reads, const gs_params *p,
                   int fetch_to_host);
int gs_result_host(gs_ctx *ctx, gs_result_view *out);
int gs_result_device(gs_ctx *ctx, gs_result_view *out);
/* Text records exactly as `seed_gen -o` prints them (seed_gen.cu:3625-3647),
 * appended to an open file descriptor; first_read_no is 1-based.  Formatted
 * on the GPU from the device result (copied out in 64 MiB chunks that overlap
 * the writes); by the host from the host result when there is no device
 * result. */
int gs_result_write_text(gs_ctx *ctx, int fd, uint32_t first_read_no, int smem);
/* The same, always formatted by the host from the host result. */
int gs_result_write_text_host(gs_ctx *ctx, int fd, uint32_t first_read_no, int smem);
/* The same text in device memory owned by the context (valid until its next
 * call): *d_text, *n_bytes.  No counterpart in the reference. */
int gs_result_text_device(gs_ctx *ctx, uint32_t first_read_no, int smem, const char **d_text,
                          uint64_t *n_bytes);
/* Stream the context runs on (a cudaStream_t). */
void *gs_ctx_stream(gs_ctx *ctx);
/* Device time (ms) of the last pass's search kernel and of the whole pass,
 * from CUDA events recorded on the context stream. */
int gs_ctx_last_timing(gs_ctx *ctx, float *search_ms, float *total_ms);
/* Work of the last pass run with count_work = 1: start-table lookups,
 * 32-byte occurrence blocks of the search, LF steps and SA samples of the
 * locate stage.  With the plain kernel the search counts are the canonical
 * containment-stopped walk (the algorithmic work); with the other kernels
 * they are the lookups those kernels execute. */
int gs_ctx_last_work(gs_ctx *ctx, uint64_t out[4]);

/* Batched search, last pass run with count_work = 1 (one pass, not
 * chunks): the walk pass's steps, its steps with a neighbour interval J, the
 * 32-byte blocks it loaded for J alone (J's bounds outside the blocks of
 * I's), the steps with J that shrank I, the walkers that started with J,
 * and the distinct 128-byte lines its steps' bounds fall in -- with this
 * occurrence table (256 rows a line) and as if blocks held 192 rows in 64
 * bytes (384 rows a line).  No counterpart in the reference: these bound
 * what another containment test or block size could save. */
int gs_ctx_last_walk_counts(gs_ctx *ctx, uint64_t out[7]);
/* Batched search (GS_KERNEL_BATCHED): candidates of the last call that the
 * start pass handed to the walk pass, and the walker buffer's capacity
 * (handed beyond it: walked in the start pass instead). */
int gs_ctx_last_walkers(gs_ctx *ctx, uint64_t *n_walkers, uint64_t *capacity);
/* Walkers the last batched pass handed to its text pass, and the room it had
 * for them (0, 0 without text mode). */
int gs_ctx_last_text_jobs(gs_ctx *ctx, uint64_t *n_jobs, uint64_t *capacity);

/* ---- autotuner ----------------------------------------------------------
 * Times the search on the first `sample` reads (device buffers) by coordinate
 * descent (two rounds) over the kernel's launch knobs -- queue_chunk and
 * ctas_per_sm for GS_KERNEL_BATCHED, those and handoff_lanes/handoff_steps
 * for GS_KERNEL_LOCKSTEP -- and writes the fastest setting into *p; *best_ms
 * gets its search time.  Results never depend on these knobs.  No
 * counterpart in the reference. */
int gs_autotune(gs_ctx *ctx, const char *d_seqs, const uint64_t *d_offsets,
                const uint32_t *d_lengths, uint32_t n_reads, gs_params *p, uint32_t sample,
                float *best_ms);

/* ---- serving (continuous batching) ------------------------------------
 * The reference seeds one file batch after another (seed_gen.cu:2910-3790).
 * A server keeps the index resident and accepts read sets at any time;
 * n_slots worker threads, each with its own stream and workspace, merge every
 * pending request that fits (arrival order, max_batch_reads, HBM budget) into
 * one pass, so passes of different slots overlap and new requests join as
 * soon as a slot and memory free up.  A request's seeds depend only on its
 * reads: the same alone or merged with others.  Many slots with small passes
 * keep the GPU busy while other slots copy and merge: at 120% of load on
 * config-3 requests, 12 slots of up to 2^18 reads sustained the device's
 * peak (43.7 M reads/s); 4 slots of 2^20, 32.8 M. */
typedef struct gs_server gs_server;
typedef struct {
    int32_t n_slots;            /* concurrent passes (default 12) */
    int32_t max_batch_reads;    /* reads merged into one pass (default 2^18) */
    uint64_t hbm_budget;        /* workspace bytes the slots may hold together (0: 60% of free) */
    gs_params params;           /* k, mode, kernel ... applied to every request */
} gs_server_opts;
typedef struct {
    uint64_t submitted, completed, failed, passes, reads, max_batch_reads;
    uint64_t pending, reserved_bytes, budget_bytes;
    /* cumulative microseconds: copying requests in (gs_server_submit), merging
     * a pass's requests into pinned memory, the pass itself (gs_seed: copies
     * and GPU), splitting its seeds back per request */
    uint64_t submit_us, merge_us, seed_us, split_us;
} gs_server_stats;
int gs_server_start(gs_index *idx, const gs_server_opts *opts, gs_server **out);
/* Copies the request's reads; the caller's buffers are free on return. */
int gs_server_submit(gs_server *srv, const char *seqs, const uint64_t *offsets,
                     const uint32_t *lengths, uint32_t n_reads, uint64_t *request_id);
/* The same without copying the bases when the reads lie back to back in
 * seqs (offsets[i+1] == offsets[i] + lengths[i]): the pass reads them from
 * the caller's buffer, which must stay unchanged until gs_server_wait
 * reports the request done.  Offsets and lengths are still copied; reads
 * that are not back to back are copied as by gs_server_submit.  For a
 * client that submits faster than one thread copies bases. */
int gs_server_submit_ref(gs_server *srv, const char *seqs, const uint64_t *offsets,
                         const uint32_t *lengths, uint32_t n_reads, uint64_t *request_id);
/* 0 when done (or the request's error), GS_ETIMEOUT after timeout_ms (< 0: wait). */
int gs_server_wait(gs_server *srv, uint64_t request_id, int32_t timeout_ms);
/* Host view of a finished request's seeds (valid until release) and its
 * submit-to-done latency. */
int gs_server_result(gs_server *srv, uint64_t request_id, gs_result_view *out, double *latency_ms);
int gs_server_release(gs_server *srv, uint64_t request_id);
int gs_server_get_stats(gs_server *srv, gs_server_stats *out);
/* Finishes the pending requests, then stops the workers. */
void gs_server_stop(gs_server *srv);
/* Load generator (no counterpart in the reference): submits request i --
 * reads first[i] .. first[i]+count[i]-1 of a pool -- gap_ms[i] after request
 * i-1, waits for all, and reports each submit-to-done latency, the wall time
 * from first submission to last completion and the submission span. */
int gs_server_replay(gs_server *srv, const char *pool_seqs, const uint64_t *pool_offsets,
                     const uint32_t *pool_lengths, uint32_t n_req, const uint32_t *first,
                     const uint32_t *count, const double *gap_ms, double *latency_ms,
                     double *wall_ms, double *submit_ms);

/* ---- allocation-free pass ---------------------------------------------
 * No counterpart in the reference.  For callers that may not allocate device
 * memory while they run (a process that fixed its HBM budget at start-up, or
 * one that cannot let cudaMalloc/cudaFree synchronise the device under other
 * streams' work): a seeding pass whose every scratch buffer lies inside one
 * static device array of GS_NOALLOC_SCRATCH_BYTES that the library keeps on
 * each GPU that loads it.  The search is the lockstep form without its
 * tail-pass hand-over (it needs no walker or hand-over buffer); the seeds,
 * positions and offsets are the same integers gs_seed_device gives.  Of
 * gs_params it reads k, smem, n_mode, lf_mode, max_occ and mem_next; kernel must be
 * GS_KERNEL_BATCHED or GS_KERNEL_LOCKSTEP, and the launch knobs are the
 * lockstep form's defaults.  It allocates nothing; the caller passes device
 * reads and device output buffers (seeds, positions, per-read offsets of
 * n_reads + 1 entries) and gets the counts in *n_seeds_out and *n_pos_out.
 * Limits per call: GS_NOALLOC_MAX_READS reads, GS_NOALLOC_MAX_SLOTS candidate
 * slots (2 per start position), seeds and positions as below; larger inputs
 * are rejected with GS_EINVAL, larger results with GS_EOVERFLOW (counts still
 * reported).  The call synchronises its stream three times to size the pass.
 * The first call on a device looks up the array's device address and keeps
 * it; make that call before any stream capture, and do not reset the device
 * (cudaDeviceReset) while the library is loaded.  Calls share the array:
 * calls that overlap on the GPU race, so serialise them. */
#define GS_NOALLOC_SCRATCH_BYTES (64u << 20)
#define GS_NOALLOC_MAX_READS 65536u
#define GS_NOALLOC_MAX_SLOTS (1u << 21)
#define GS_NOALLOC_MAX_SEEDS (1u << 20)
#define GS_NOALLOC_MAX_POS (1u << 22)
int gs_seed_noalloc(gs_index *idx, const char *d_seqs, const uint64_t *d_offsets,
                    const uint32_t *d_lengths, uint32_t n_reads, const gs_params *p,
                    void *cuda_stream, gs_seed_rec *d_seeds, uint64_t seed_cap, uint32_t *d_pos,
                    uint64_t pos_cap, uint64_t *d_read_seed_off, uint64_t *d_read_pos_off,
                    uint64_t *n_seeds_out, uint64_t *n_pos_out);

/* ---- errors ------------------------------------------------------------- */
const char *gs_last_error(void);
const char *gs_strerror(int code);
int gs_version(void);

#ifdef __cplusplus
}
#endif
#endif
