/*
 * gs_internal.h -- device data layout and helpers shared by the kernels.
 */
#ifndef GS_INTERNAL_H
#define GS_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/gpuseed.h"

#define GS_OCC_INTERVAL 64u   /* rows per occurrence block (seed_gen.cu:29) */
#define GS_BLOCK_WORDS 8u     /* 4 counts + 4 bit-slice words of 64 bases = 32 bytes */
#define GS_K0 13              /* k-mer table length (seed_gen.cu:2822) */
#define GS_HIST 8             /* containment history depth of the batched search */
#define GS_CHUNK 31           /* candidates owned by one warp work item */
#define GS_PCHUNK 30          /* read positions owned by one paired work item */
#define GS_HANDOFF_LANES 2    /* default hand-over threshold of the batched search */
#define GS_HANDOFF_STEPS 4
#define GS_QUEUE_CHUNK 4      /* default work items per queue grab */

/* Device view of the index, passed by value to every kernel.
 * occ: one 32-byte block per 64 rows of the $-removed BWT string:
 *      {count of A, C, G, T before the block, H0, H1, L0, L1}: the high and
 *      low bits of the block's 64 bases, base i at bit 31 - (i & 31) of
 *      word i >> 5 (gs_fm.cuh).
 * sa:  sampled suffix array, sa[0] = 0xffffffff (the $ row).
 * kmer: (l,u) of every 13-mer, base j at bits 2j, processed first.
 * Optional text structures, all built from occ and sa in HBM:
 * saf:  the full suffix array, saf[row] for every row 0..seq_len (saf[0] =
 *       0xffffffff like sa[0]);
 * text: the reference text T[0..seq_len), 16 bases per word, base i at bits
 *       2*(i & 15) of word i >> 4, padded by two zero words;
 * isa:  the row of the suffix at text position j * GS_ISA_STEP, for every
 *       j * GS_ISA_STEP <= seq_len;
 * quirk_lo / quirk_n: text positions [quirk_lo, quirk_lo + quirk_n) are the
 *       rows whose LF walk passes row primary+1 before a sampled row; the LF
 *       quirk locates them at position - quirk_lo;
 * text_min: a walker that has taken this many steps with a one-row interval
 *       and no neighbour interval, with 16 or more bases left, compares the
 *       read with the text (0: never). */
#define GS_ISA_STEP 2u
#define GS_TEXT_MARK 0xf0000000u     /* jl of a text-mode walker */
#define GS_REGIME_MARK 0xe0000000u   /* jl (+ steps) of a one-row walker without J */
struct GsDevIndex {
    const uint32_t *occ;
    const uint32_t *sa;
    const uint2 *kmer;
    const uint4 *kmerx;        /* optional table of all kx-mers, same bit order: x,y the
                                * packed entry of X, z,w that of X's reverse complement */
    const uint32_t *saf;
    const uint32_t *text;
    const uint32_t *isa;
    int32_t kx;                /* 14..16, or 0 when there is no longer table */
    uint32_t primary, seq_len, sa_intv, n_sa;
    uint32_t L2[5];
    uint32_t quirk_lo, quirk_n;
    int32_t text_min;
};

/* Candidate slot written by the search kernels; y == 0 marks "no record". */
struct GsRec {
    int32_t x, y;
    uint32_t l, u;
};

/* A candidate handed from the lockstep search to the tail pass. */
struct GsCont {
    uint32_t r;
    int32_t anchor, pos;
    uint32_t l, u;
    uint32_t fwd;
};

/* A candidate that survived its start in the batched search: its interval
 * I = [l,u] at the start's far end (anchor -/+ start length - 1) and
 * J = [jl,ju] (jl > ju: none), the interval of the same string extended by
 * one base toward the longer match (the neighbour candidate's string at the
 * same far end) -- or, with the pending flag, the neighbour's own start
 * interval, one base short of that far end.  24 bytes. */
struct __align__(8) GsWalker {
    uint32_t r;
    uint32_t anchor;    /* bits 0-29: anchor; bit 30: J pending; bit 31: forward strand */
    uint32_t l, u, jl, ju;
};

/* Per-batch device arguments shared by the pipeline kernels. */
struct GsBatch {
    const char *seqs;          /* ASCII bases */
    const uint64_t *offsets;   /* per read */
    const uint32_t *lengths;   /* per read */
    uint32_t n_reads;
    int32_t k, smem, n_mode, lf_mode;
    uint64_t *slot_off;        /* per read (n+1): first candidate slot */
    uint32_t *item_off;        /* per read (n+1): first work item */
    GsRec *slots;              /* 2 * candidates; only slots holding a record are written */
    uint32_t *recmask;         /* one bit per slot: the slot holds a record (zeroed per pass) */
    uint32_t *hist;            /* plain kernel: one word per base */
    uint32_t *rd_nf, *rd_nr;   /* per read: compacted record counts */
    uint64_t *rd_nseeds, *rd_npos;   /* per read counts ... */
    uint64_t *seed_off, *pos_off;    /* ... and their exclusive scans (n+1) */
    gs_seed_rec *seeds;            /* output seeds */
    uint64_t *seed_pos;        /* per output seed: index of its first position */
    uint32_t *pos;             /* output positions */
    uint32_t *pmap;            /* position -> seed */
    uint64_t seed_cap, pos_cap;   /* output capacities (entries) */
    uint64_t slot_cap;             /* candidate slots allocated */
    uint32_t item_cap;             /* work items the hand-over buffer is sized for */
    uint64_t cont_cap;             /* hand-over records allocated */
    uint32_t *queue;           /* [0]: work-queue head, [1]: status flags,
                                  [2]: hand-over count, [3]: tail-pass head,
                                  [4]: text jobs queued (8 words, zeroed per pass) */
    unsigned long long *work;  /* NULL or [kmer, occ blocks, lf steps, sa samples] */
    GsCont *cont;              /* NULL: no hand-over; else n_items * handoff_lanes entries */
    int32_t handoff_lanes;     /* hand over when at most this many owned lanes extend ... */
    int32_t handoff_steps;     /* ... after at least this many lockstep steps */
    uint32_t max_occ;          /* 0 or the largest interval an output seed may have */
    int32_t mem_next;          /* GS_MEM_NEXT_READ | GS_MEM_NEXT_GPUSEED (MEM mode) */
    int32_t paired;            /* batched start pass: work items of read positions, one
                                * table entry for both strands' candidates (set by
                                * gs_launch_prepare) */
    GsWalker *walkers;         /* batched search: survivors of the start pass */
    uint64_t walker_cap;       /* entries allocated (0: every walk is left to the leftover pass) */
    uint32_t walker_chunk;     /* entries a start-pass warp reserves at a time */
    struct GsTextJob *text_jobs;   /* walkers handed to the text pass */
    uint64_t text_cap;         /* entries allocated (0: text mode stays inline) */
};

/* A walker that entered text mode in the walk pass, finished by the text
 * pass: its read, anchor (| GS_WALKER_FWD), far end and row. */
struct GsTextJob {
    uint32_t r, anchor, pos, l;
};

#define GS_FLAG_WALK 1u
#define GS_FLAG_OVERFLOW 2u
#define GS_FLAG_LEFTOVER 4u   /* the start pass left walks in record slots (leftover pass) */

__host__ __device__ static inline uint32_t gs_fwd_code(unsigned char ch)
{
    /* pack_4bit_fow table (seed_gen.cu:2539): A0 C1 G2 T3 N4, others 0/5 */
    return (0x24031005u >> ((ch & 7u) << 2)) & 15u;
}

__host__ __device__ static inline uint32_t gs_comp_code(unsigned char ch)
{
    /* pack_4bit_rev table (seed_gen.cu:2561): complement codes */
    return (0x14002035u >> ((ch & 7u) << 2)) & 15u;
}

/* Device result as the text formatter reads it (gs_text.cu). */
struct GsTextArgs {
    uint32_t n_reads;
    uint64_t n_seeds, n_pos;
    const uint64_t *seed_off, *pos_off;   /* per read (n+1) */
    const gs_seed_rec *seeds;
    const uint64_t *seed_pos;             /* per seed: its first position */
    const uint32_t *pmap, *pos;           /* per position: its seed, its value */
    uint32_t first_read_no;
    int32_t smem;
    uint32_t *sread;                      /* per seed: its read (written) */
    uint64_t *off;                        /* per token + 1: lengths, then byte offsets */
    char *text;
};

/* host helpers (gs_api.cu) */
void gs_set_error(const char *fmt, ...);
int gs_cuda_fail(cudaError_t e, const char *what);
#define GS_CUDA(call)                                         \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return gs_cuda_fail(_e, #call); \
    } while (0)

/* Makes a device current for the rest of the scope and gives the calling
 * thread its previous current device back on every return path, so that a
 * library call does not leave a C caller that drives several GPUs from one
 * thread on another device. */
struct GsDeviceGuard {
    int prev = -1;
    bool changed = false;
    cudaError_t enter(int dev)
    {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return e;
        if (prev == dev) return cudaSuccess;
        e = cudaSetDevice(dev);
        changed = e == cudaSuccess;
        return e;
    }
    ~GsDeviceGuard()
    {
        if (changed) cudaSetDevice(prev);
    }
};
#define GS_ON_DEVICE(dev)            \
    GsDeviceGuard gs_device_guard_;  \
    GS_CUDA(gs_device_guard_.enter(dev))

/* kernel launchers (defined next to their kernels) */
int gs_build_kmer_table(const GsDevIndex &idx, uint2 *table, cudaStream_t st);
int gs_launch_text_lengths(const GsTextArgs &a, cudaStream_t st);
int gs_launch_text_write(const GsTextArgs &a, cudaStream_t st);
int gs_build_kmerx_table(const GsDevIndex &idx, uint4 *table, int kx, cudaStream_t st);
/* full SA, text and sampled ISA from occ + sa; GS_EFORMAT when the index
 * does not describe one text (the structures are then not used) */
int gs_build_text(GsDevIndex &idx, uint32_t *saf, uint32_t *text, uint32_t *isa, cudaStream_t st);
/* n_items: host-known work-item count for grid sizing, or 0 (graph capture):
 * the kernels read the count from item_off[n_reads] on the device */
int gs_launch_search(const GsDevIndex &idx, GsBatch &b, int kernel, int queue_chunk,
                     int ctas_per_sm, uint32_t n_items, cudaStream_t st);
int gs_launch_prepare(const GsDevIndex &I, GsBatch &b, int kernel, cudaStream_t st);
int gs_launch_finalize_count(const GsDevIndex &idx, GsBatch &b, cudaStream_t st);
int gs_launch_finalize_emit(const GsDevIndex &idx, GsBatch &b, cudaStream_t st);
/* n_seeds / n_pos: host-known totals, or 0 to size the grids by the
 * capacities and read the totals on the device (graph capture) */
int gs_launch_locate(const GsDevIndex &idx, GsBatch &b, uint64_t n_seeds, uint64_t n_pos,
                     cudaStream_t st);

#endif
