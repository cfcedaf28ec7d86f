/*
 * gs_api.cu -- seeding context: workspace, the per-batch pipeline, results,
 * text records and error reporting.
 *
 * One gs_seed* call does for one batch what the body of seed_gen's batch loop
 * does (seed_gen.cu:2910-3790), on one stream, with the workspace kept across
 * calls instead of ~15 cudaMalloc/cudaFree per batch (:3029-3102,
 * :3750-3770):
 *
 *   prepare  -> slot / work-item counts per read, exclusive scans
 *   search   -> one record slot per candidate (gs_search.cu)
 *   count    -> per-read compaction + filter counts (gs_post.cu)
 *   scan     -> seed / position offsets
 *   emit     -> output seeds in output order
 *   locate   -> positions by the sampled-SA walk
 */
#include "gs_internal.h"

#define GS_SEED_CHUNK_READS (1u << 22)   /* gs_seed runs batches of this or more in chunks:
                                            the middle ones of about this many reads */
#define GS_SEED_END_FRACTION 0.1         /* the first and the last chunk, of a middle one */
#define GS_SEED_MAX_CHUNKS 16

#include <cub/cub.cuh>

#include <atomic>

#include <errno.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------ */
/* errors */

static thread_local char g_err[512];

void gs_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int gs_cuda_fail(cudaError_t e, const char *what)
{
    gs_set_error("%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return GS_ENOMEM;
    }
    return GS_ECUDA;
}

extern "C" const char *gs_last_error(void) { return g_err; }

extern "C" const char *gs_strerror(int code)
{
    switch (code) {
    case GS_OK: return "ok";
    case GS_EINVAL: return "invalid argument";
    case GS_EIO: return "i/o error";
    case GS_EFORMAT: return "index format error";
    case GS_ENOMEM: return "out of memory";
    case GS_ECUDA: return "CUDA error";
    case GS_EWALK: return "sampled-SA walk exceeded its limit";
    case GS_EOVERFLOW: return "output capacity exceeded";
    case GS_ETIMEOUT: return "bounded wait ran out";
    case GS_ESTATE: return "invalid state";
    default: return "unknown error";
    }
}

extern "C" int gs_version(void) { return 100; }

/* ------------------------------------------------------------------ */
/* index accessors (gs_index.cu) */

const GsDevIndex *gs_index_dev(const gs_index *idx);
int gs_index_device(const gs_index *idx);
uint32_t gs_index_generation(const gs_index *idx);
float gs_index_l2_ratio(const gs_index *idx);
size_t gs_index_occ_bytes(const gs_index *idx);

/* ------------------------------------------------------------------ */
/* context */

/* Workspace growth is stream-ordered (the device's default memory pool):
 * cudaFree would wait for the whole device, stalling every other context's
 * work -- the serving loop's slots grow their workspaces while the others
 * run. */
template <class T>
static int grow(T *&p, size_t &cap, size_t n, cudaStream_t st)
{
    if (n <= cap && p) return GS_OK;
    size_t nc = n + n / 4 + 64;
    T *np = NULL;
    cudaError_t e = cudaMallocAsync((void **)&np, nc * sizeof(T), st);
    if (e != cudaSuccess) return gs_cuda_fail(e, "cudaMallocAsync(workspace)");
    if (p) cudaFreeAsync(p, st);
    p = np;
    cap = nc;
    return GS_OK;
}

/* One chunk of a gs_seed batch: where its results go in the batch's host
 * arrays, and what it found. */
struct GsChunkOut {
    uint32_t first_read;      /* the chunk's first read in the batch */
    uint64_t base_s, base_p;  /* seeds and positions of the chunks before it */
    double scale;             /* batch reads / chunk reads, to size the host arrays once */
    int wait_d2h;             /* the previous chunk's copy-out may still run */
    uint64_t n_seeds, n_pos;  /* out */
};

template <class T>
static int grow_host(T *&p, size_t &cap, size_t n)
{
    if (n <= cap && p) return GS_OK;
    size_t nc = n + n / 4 + 64;
    T *np = NULL;
    cudaError_t e = cudaMallocHost(&np, nc * sizeof(T));
    if (e != cudaSuccess) return gs_cuda_fail(e, "cudaMallocHost(result)");
    cudaFreeHost(p);
    p = np;
    cap = nc;
    return GS_OK;
}

/* grow_host keeping the first `keep` entries, once the copies on `busy`
 * that write into the old array are done */
template <class T>
static int grow_host_keep(T *&p, size_t &cap, size_t n, size_t keep, cudaStream_t busy)
{
    if (n <= cap && p) return GS_OK;
    GS_CUDA(cudaStreamSynchronize(busy));
    size_t nc = n + n / 4 + 64;
    T *np = NULL;
    cudaError_t e = cudaMallocHost(&np, nc * sizeof(T));
    if (e != cudaSuccess) return gs_cuda_fail(e, "cudaMallocHost(result)");
    if (keep && p) memcpy(np, p, keep * sizeof(T));
    cudaFreeHost(p);
    p = np;
    cap = nc;
    return GS_OK;
}

struct gs_ctx {
    gs_index *idx;
    cudaStream_t st;
    bool own_stream;
    cudaEvent_t ev0, ev_s0, ev_s1, ev1;
    cudaStream_t st_copy;       /* copies seeds out while positions are located */
    cudaEvent_t ev_emit;
    /* gs_seed in chunks: reads go up on st_h2d, each chunk's results come
     * down on st_copy while the next chunk runs on st */
    cudaStream_t st_h2d;
    cudaEvent_t ev_h2d[GS_SEED_MAX_CHUNKS];
    cudaEvent_t ev_done, ev_d2h;
    /* inputs staged by gs_seed_rec */
    char *d_seqs; size_t cap_seqs;
    uint64_t *d_offsets; size_t cap_offsets;
    uint32_t *d_lengths; size_t cap_lengths;
    /* per read */
    uint64_t *slot_cnt, *slot_off; size_t cap_slot_cnt, cap_slot_off;
    uint32_t *item_cnt, *item_off; size_t cap_item_cnt, cap_item_off;
    uint32_t *rd_nf, *rd_nr; size_t cap_nf, cap_nr;
    uint64_t *rd_nseeds, *rd_npos; size_t cap_rns, cap_rnp;
    uint64_t *seed_off, *pos_off; size_t cap_so, cap_po;
    /* per candidate / base / output */
    GsRec *slots; size_t cap_slots;
    uint32_t *recmask; size_t cap_recmask;
    uint32_t *hist; size_t cap_hist;
    gs_seed_rec *seeds; size_t cap_seeds;
    uint64_t *seed_pos; size_t cap_seed_pos;
    uint32_t *pos; size_t cap_pos;
    uint32_t *pmap; size_t cap_pmap;
    GsCont *cont; size_t cap_cont;
    GsWalker *walkers; size_t cap_walkers;
    GsTextJob *text_jobs; size_t cap_text_jobs;
    uint64_t last_text_cap, last_text_jobs;
    /* text formatting on the GPU */
    uint32_t *t_sread; size_t cap_t_sread;
    uint64_t *t_off; size_t cap_t_off;
    char *t_text; size_t cap_t_text;
    char *h_text[2];            /* pinned copy-out buffers */
    cudaEvent_t t_ev[2];
    uint64_t last_walkers, last_walker_cap;
    uint32_t walker_per16;      /* automatic walker-buffer size, per 16 work items */
    uint32_t *queue;
    uint64_t *d_max;
    unsigned long long *d_work;
    uint64_t work[4];
    uint64_t walk_counts[7];   /* count_work pass: gs_ctx_last_walk_counts */
    void *cub_tmp; size_t cap_cub;
    uint64_t *h_small;          /* pinned scalars */
    /* host result */
    uint64_t *h_seed_off; size_t cap_h_so;
    uint64_t *h_pos_off; size_t cap_h_po;
    gs_seed_rec *h_seeds; size_t cap_h_seeds;
    uint32_t *h_pos; size_t cap_h_pos;
    uint32_t n_reads;
    uint64_t n_seeds, n_pos;
    int have_host, have_dev;
    float t_search, t_total;
    /* captured pass */
    cudaGraphExec_t gexec;
    const char *g_seqs;
    const uint64_t *g_offs;
    const uint32_t *g_lens;
    uint32_t g_n;
    uint32_t g_gen;   /* index generation the graph was captured with */
    gs_params g_params;
    uint32_t g_items;
};

extern "C" int gs_ctx_create(gs_index *idx, void *cuda_stream, gs_ctx **out)
{
    if (!idx || !out) return GS_EINVAL;
    *out = NULL;
    GS_ON_DEVICE(gs_index_device(idx));
    gs_ctx *c = (gs_ctx *)calloc(1, sizeof(gs_ctx));
    if (!c) return GS_ENOMEM;
    c->idx = idx;
    cudaError_t e = cudaSuccess;
    if (cuda_stream) {
        c->st = (cudaStream_t)cuda_stream;
    } else {
        e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
        c->own_stream = true;
    }
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_s0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_s1);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st_copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_emit, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st_h2d, cudaStreamNonBlocking);
    for (int i = 0; i < GS_SEED_MAX_CHUNKS && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&c->ev_h2d[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_d2h, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&c->queue, 32);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_max, 16);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_work, 128);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_small, 256);
    if (e != cudaSuccess) {
        int rc = gs_cuda_fail(e, "gs_ctx_create");
        gs_ctx_free(c);
        return rc;
    }
    /* The persisting-L2 carve-out is a limit of the whole CUDA context: once
     * a context of this process set it, it stays until reset.  On the
     * search's random accesses it costs time (70.9 -> 94.4 ms on 4M reads of
     * a 3.1 Gbp index), so a context made with the window off releases it. */
    static std::atomic<bool> persisting_set(false);   /* contexts are made from many threads */
    float ratio = gs_index_l2_ratio(idx);
    if (ratio <= 0.f && persisting_set.exchange(false)) {
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
        cudaCtxResetPersistingL2Cache();
        cudaGetLastError();
    }
    if (ratio > 0.f) {
        int dev = gs_index_device(idx), maxwin = 0, persist = 0;
        cudaDeviceGetAttribute(&maxwin, cudaDevAttrMaxAccessPolicyWindowSize, dev);
        cudaDeviceGetAttribute(&persist, cudaDevAttrMaxPersistingL2CacheSize, dev);
        if (maxwin > 0 && persist > 0) {
            size_t occ = gs_index_occ_bytes(idx);
            size_t win = occ < (size_t)maxwin ? occ : (size_t)maxwin;
            cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)persist);
            persisting_set.store(true);
            cudaStreamAttrValue v;
            memset(&v, 0, sizeof(v));
            v.accessPolicyWindow.base_ptr = (void *)gs_index_dev(idx)->occ;
            v.accessPolicyWindow.num_bytes = win;
            v.accessPolicyWindow.hitRatio = ratio;
            v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
            v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
            cudaStreamSetAttribute(c->st, cudaStreamAttributeAccessPolicyWindow, &v);
            cudaGetLastError();
        }
    }
    *out = c;
    return GS_OK;
}

extern "C" void gs_ctx_free(gs_ctx *c)
{
    if (!c) return;
    if (c->st) cudaStreamSynchronize(c->st);
    cudaFree(c->d_seqs); cudaFree(c->d_offsets); cudaFree(c->d_lengths);
    cudaFree(c->slot_cnt); cudaFree(c->slot_off); cudaFree(c->item_cnt); cudaFree(c->item_off);
    cudaFree(c->rd_nf); cudaFree(c->rd_nr); cudaFree(c->rd_nseeds); cudaFree(c->rd_npos);
    cudaFree(c->seed_off); cudaFree(c->pos_off);
    cudaFree(c->slots); cudaFree(c->hist); cudaFree(c->seeds); cudaFree(c->seed_pos);
    cudaFree(c->pos); cudaFree(c->pmap); cudaFree(c->queue); cudaFree(c->d_max);
    cudaFree(c->cont);
    cudaFree(c->walkers);
    cudaFree(c->text_jobs);
    cudaFree(c->recmask);
    cudaFree(c->t_sread); cudaFree(c->t_off); cudaFree(c->t_text);
    cudaFreeHost(c->h_text[0]); cudaFreeHost(c->h_text[1]);
    if (c->t_ev[0]) cudaEventDestroy(c->t_ev[0]);
    if (c->t_ev[1]) cudaEventDestroy(c->t_ev[1]);
    cudaFree(c->d_work);
    cudaFree(c->cub_tmp);
    cudaFreeHost(c->h_small);
    cudaFreeHost(c->h_seed_off); cudaFreeHost(c->h_pos_off);
    cudaFreeHost(c->h_seeds); cudaFreeHost(c->h_pos);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev_s0) cudaEventDestroy(c->ev_s0);
    if (c->ev_s1) cudaEventDestroy(c->ev_s1);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev_emit) cudaEventDestroy(c->ev_emit);
    if (c->st_copy) {
        cudaStreamSynchronize(c->st_copy);
        cudaStreamDestroy(c->st_copy);
    }
    if (c->st_h2d) {
        cudaStreamSynchronize(c->st_h2d);
        cudaStreamDestroy(c->st_h2d);
    }
    for (int i = 0; i < GS_SEED_MAX_CHUNKS; i++)
        if (c->ev_h2d[i]) cudaEventDestroy(c->ev_h2d[i]);
    if (c->ev_done) cudaEventDestroy(c->ev_done);
    if (c->ev_d2h) cudaEventDestroy(c->ev_d2h);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->own_stream && c->st) cudaStreamDestroy(c->st);
    free(c);
}

extern "C" void *gs_ctx_stream(gs_ctx *c) { return c ? (void *)c->st : NULL; }

extern "C" int gs_ctx_last_work(gs_ctx *c, uint64_t out[4])
{
    if (!c || !out) return GS_EINVAL;
    memcpy(out, c->work, sizeof(c->work));
    return GS_OK;
}

extern "C" int gs_ctx_last_walk_counts(gs_ctx *c, uint64_t out[7])
{
    if (!c || !out) return GS_EINVAL;
    memcpy(out, c->walk_counts, sizeof(c->walk_counts));
    return GS_OK;
}

extern "C" int gs_ctx_last_walkers(gs_ctx *c, uint64_t *n_walkers, uint64_t *capacity)
{
    if (!c) return GS_EINVAL;
    if (n_walkers) *n_walkers = c->last_walkers;
    if (capacity) *capacity = c->last_walker_cap;
    return GS_OK;
}

extern "C" int gs_ctx_last_text_jobs(gs_ctx *c, uint64_t *n_jobs, uint64_t *capacity)
{
    if (!c) return GS_EINVAL;
    if (n_jobs) *n_jobs = c->last_text_jobs;
    if (capacity) *capacity = c->last_text_cap;
    return GS_OK;
}

extern "C" int gs_ctx_last_timing(gs_ctx *c, float *search_ms, float *total_ms)
{
    if (!c) return GS_EINVAL;
    if (search_ms) *search_ms = c->t_search;
    if (total_ms) *total_ms = c->t_total;
    return GS_OK;
}

/* end of the longest read, for the plain kernel's per-base history; out[1]
 * becomes non-zero when a read does not end at or before the next one's
 * start (gs_seed then copies the reads up whole, not in chunks) */
__global__ void gs_max_end_kernel(const uint64_t *off, const uint32_t *len, uint32_t n,
                                  unsigned long long *out)
{
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long e = r < n ? (unsigned long long)(off[r] + len[r]) : 0ull;
    const bool disorder = r + 1 < n && e > off[r + 1];
    if (__any_sync(0xffffffffu, disorder) && (threadIdx.x & 31) == 0) atomicOr(&out[1], 1ull);
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long t = __shfl_xor_sync(0xffffffffu, e, o);
        e = t > e ? t : e;
    }
    if ((threadIdx.x & 31) == 0 && e) atomicMax(out, e);
}

/* Device scalars into the pinned scalar block, written by a kernel: pinned
 * host memory is mapped into the device's address space under unified
 * addressing, and a read that takes no copy engine never queues behind a
 * large copy-out on another stream. */
__global__ void gs_fetch_small_kernel(uint32_t *dst, const uint32_t *src, uint32_t n_words)
{
    if (threadIdx.x < n_words) dst[threadIdx.x] = src[threadIdx.x];
}

static int fetch_small(uint64_t *dst, const void *src, size_t bytes, cudaStream_t st)
{
    gs_fetch_small_kernel<<<1, 32, 0, st>>>((uint32_t *)dst, (const uint32_t *)src,
                                            (uint32_t)(bytes / 4));
    GS_CUDA(cudaGetLastError());
    return GS_OK;
}

/* a chunk's per-read offsets made batch-wide */
__global__ void gs_add_base_kernel(uint64_t *seed_off, uint64_t *pos_off, uint32_t n, uint64_t bs,
                                   uint64_t bp)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        seed_off[i] += bs;
        pos_off[i] += bp;
    }
}

template <class In, class Out>
static int exclusive_scan(gs_ctx *c, In in, Out out, size_t n)
{
    size_t bytes = 0;
    GS_CUDA(cub::DeviceScan::ExclusiveSum(NULL, bytes, in, out, (int64_t)n, c->st));
    if (bytes > c->cap_cub) {
        if (c->cub_tmp) cudaFreeAsync(c->cub_tmp, c->st);
        c->cub_tmp = NULL;
        c->cap_cub = 0;
        GS_CUDA(cudaMallocAsync(&c->cub_tmp, bytes, c->st));
        c->cap_cub = bytes;
    }
    GS_CUDA(cub::DeviceScan::ExclusiveSum(c->cub_tmp, bytes, in, out, (int64_t)n, c->st));
    return GS_OK;
}

static int check_params(const gs_params *p)
{
    if (!p) {
        gs_set_error("null gs_params");
        return GS_EINVAL;
    }
    if (p->k < GS_K0 || p->k > 1000000) {
        gs_set_error("min seed length k=%d outside [%d, 1000000]: below 13 the 13-mer lookup "
                     "would read before the read",
                     p->k, GS_K0);
        return GS_EINVAL;
    }
    if ((p->n_mode != GS_N_WILDCARD && p->n_mode != GS_N_STOP) ||
        (p->lf_mode != GS_LF_GPUSEED && p->lf_mode != GS_LF_BWA) ||
        (p->kernel != GS_KERNEL_BATCHED && p->kernel != GS_KERNEL_PLAIN &&
         p->kernel != GS_KERNEL_LOCKSTEP) ||
        (p->mem_next != GS_MEM_NEXT_READ && p->mem_next != GS_MEM_NEXT_GPUSEED)) {
        gs_set_error("gs_params mode out of range");
        return GS_EINVAL;
    }
    return GS_OK;
}

#define RC(x)                    \
    do {                         \
        int _rc = (x);           \
        if (_rc) return _rc;     \
    } while (0)

/* One pass over n_reads device-resident reads.  fetch: copy the result to
 * the context's host arrays.  co (gs_seed's chunks): instead, copy this
 * chunk's result into the batch's host arrays on st_copy, batch-wide, and
 * return without waiting for that copy. */
static int run_pipeline(gs_ctx *c, const char *d_seqs, const uint64_t *d_offsets,
                        const uint32_t *d_lengths, uint32_t n_reads, const gs_params *p,
                        int fetch, GsChunkOut *co = NULL)
{
    const GsDevIndex &I = *gs_index_dev(c->idx);
    cudaStream_t st = c->st;
    c->have_host = c->have_dev = 0;
    c->n_reads = n_reads;
    size_t nr1 = (size_t)n_reads + 1;
    RC(grow(c->slot_cnt, c->cap_slot_cnt, nr1, c->st));
    RC(grow(c->slot_off, c->cap_slot_off, nr1, c->st));
    RC(grow(c->item_cnt, c->cap_item_cnt, nr1, c->st));
    RC(grow(c->item_off, c->cap_item_off, nr1, c->st));
    RC(grow(c->rd_nf, c->cap_nf, nr1, c->st));
    RC(grow(c->rd_nr, c->cap_nr, nr1, c->st));
    RC(grow(c->rd_nseeds, c->cap_rns, nr1, c->st));
    RC(grow(c->rd_npos, c->cap_rnp, nr1, c->st));
    RC(grow(c->seed_off, c->cap_so, nr1, c->st));
    RC(grow(c->pos_off, c->cap_po, nr1, c->st));

    GsBatch B;
    memset(&B, 0, sizeof(B));
    B.seqs = d_seqs;
    B.offsets = d_offsets;
    B.lengths = d_lengths;
    B.n_reads = n_reads;
    B.k = p->k;
    B.smem = p->smem ? 1 : 0;
    B.n_mode = p->n_mode;
    B.lf_mode = p->lf_mode;
    B.max_occ = p->max_occ > 0 ? (uint32_t)p->max_occ : 0u;
    B.mem_next = p->mem_next;
    B.queue = c->queue;
    B.work = p->count_work ? c->d_work : NULL;
    memset(c->work, 0, sizeof(c->work));
    memset(c->walk_counts, 0, sizeof(c->walk_counts));

    GS_CUDA(cudaEventRecord(c->ev0, st));
    if (B.work) GS_CUDA(cudaMemsetAsync(c->d_work, 0, 128, st));
    GS_CUDA(cudaMemsetAsync(c->queue, 0, 32, st));
    B.slot_off = c->slot_cnt;
    B.item_off = c->item_cnt;
    RC(gs_launch_prepare(I, B, p->kernel, st));
    RC(exclusive_scan(c, c->slot_cnt, c->slot_off, nr1));
    RC(exclusive_scan(c, c->item_cnt, c->item_off, nr1));
    B.slot_off = c->slot_off;
    B.item_off = c->item_off;
    RC(fetch_small(&c->h_small[0], c->slot_off + n_reads, 8, st));
    RC(fetch_small(&c->h_small[1], c->item_off + n_reads, 4, st));
    if (p->kernel == GS_KERNEL_PLAIN) {
        GS_CUDA(cudaMemsetAsync(c->d_max, 0, 8, st));
        if (n_reads)
            gs_max_end_kernel<<<(n_reads + 255) / 256, 256, 0, st>>>(
                d_offsets, d_lengths, n_reads, (unsigned long long *)c->d_max);
        RC(fetch_small(&c->h_small[2], c->d_max, 8, st));
    }
    GS_CUDA(cudaStreamSynchronize(st));
    uint64_t n_slots = c->h_small[0];
    uint32_t n_items = (uint32_t)(c->h_small[1] & 0xffffffffu);
    RC(grow(c->slots, c->cap_slots, n_slots + 1, c->st));
    RC(grow(c->recmask, c->cap_recmask, (c->cap_slots + 31) / 32 + 1, c->st));
    B.slots = c->slots;
    B.slot_cap = c->cap_slots;
    B.recmask = c->recmask;
    GS_CUDA(cudaMemsetAsync(c->recmask, 0, ((n_slots + 31) / 32 + 1) * sizeof(uint32_t), st));
    B.item_cap = n_items;
    if (p->kernel == GS_KERNEL_PLAIN) {
        RC(grow(c->hist, c->cap_hist, c->h_small[2] + 1, c->st));
        B.hist = c->hist;
    } else if (p->kernel == GS_KERNEL_LOCKSTEP && p->handoff_lanes >= 0) {
        B.handoff_lanes = p->handoff_lanes ? p->handoff_lanes : GS_HANDOFF_LANES;
        B.handoff_steps = p->handoff_steps > 0 ? p->handoff_steps : GS_HANDOFF_STEPS;
        if (B.handoff_lanes > 32) B.handoff_lanes = 32;
        RC(grow(c->cont, c->cap_cont, (size_t)n_items * (size_t)B.handoff_lanes + 1, c->st));
        B.cont = c->cont;
        B.cont_cap = c->cap_cont;
    }
    c->last_walker_cap = 0;
    c->last_text_cap = 0;
    if (p->kernel == GS_KERNEL_BATCHED && p->walker_slots >= 0) {
        /* entries per 16 work items of 31 candidates (a paired item of 30
         * windows counts as two): as asked, or automatic -- 16 per item
         * with a start table (forced codes settle most candidates), all 31
         * without, and 1.5x more after a pass that filled its buffer */
        if (!c->walker_per16) c->walker_per16 = I.kx > GS_K0 ? 256u : 512u;
        const uint64_t per16 = p->walker_slots ? (uint64_t)p->walker_slots : c->walker_per16;
        const uint64_t units = (uint64_t)n_items * (B.paired ? 2u : 1u);
        uint64_t want = (units * per16 + 15u) / 16u + 32u;
        if (want > (1ull << 31)) want = 1ull << 31;   /* 32-bit buffer counter */
        RC(grow(c->walkers, c->cap_walkers, (size_t)want, c->st));
        B.walkers = c->walkers;
        B.walker_cap = want;
        c->last_walker_cap = want;
        /* walkers handed to the text pass: two per work item is far above
         * what reads with a few differences per 100 bases need; without
         * room a walker walks on in the walk pass */
        if (I.text_min) {
            uint64_t tw = units * 2u + 64u;
            if (tw > (1ull << 31)) tw = 1ull << 31;
            RC(grow(c->text_jobs, c->cap_text_jobs, (size_t)tw, c->st));
            B.text_jobs = c->text_jobs;
            B.text_cap = tw;
            c->last_text_cap = tw;
        }
    }

    GS_CUDA(cudaEventRecord(c->ev_s0, st));
    RC(gs_launch_search(I, B, p->kernel, p->queue_chunk, p->ctas_per_sm, n_items, st));
    GS_CUDA(cudaEventRecord(c->ev_s1, st));
    /* the previous chunk's results are copied out of the buffers below while
     * this chunk searched */
    if (co && co->wait_d2h) GS_CUDA(cudaStreamWaitEvent(st, c->ev_d2h, 0));

    B.rd_nf = c->rd_nf;
    B.rd_nr = c->rd_nr;
    B.rd_nseeds = c->rd_nseeds;
    B.rd_npos = c->rd_npos;
    GS_CUDA(cudaMemsetAsync(c->rd_nseeds + n_reads, 0, 8, st));
    GS_CUDA(cudaMemsetAsync(c->rd_npos + n_reads, 0, 8, st));
    RC(gs_launch_finalize_count(I, B, st));
    RC(exclusive_scan(c, c->rd_nseeds, c->seed_off, nr1));
    RC(exclusive_scan(c, c->rd_npos, c->pos_off, nr1));
    RC(fetch_small(&c->h_small[3], c->seed_off + n_reads, 8, st));
    RC(fetch_small(&c->h_small[4], c->pos_off + n_reads, 8, st));
    GS_CUDA(cudaStreamSynchronize(st));
    uint64_t n_seeds = c->h_small[3], n_pos = c->h_small[4];
    if (n_pos > 0xffffffffull * 4) {
        gs_set_error("batch emits %llu positions; split the batch", (unsigned long long)n_pos);
        return GS_EOVERFLOW;
    }
    RC(grow(c->seeds, c->cap_seeds, n_seeds + 1, c->st));
    RC(grow(c->seed_pos, c->cap_seed_pos, n_seeds + 1, c->st));
    RC(grow(c->pos, c->cap_pos, n_pos + 1, c->st));
    RC(grow(c->pmap, c->cap_pmap, n_pos + 1, c->st));
    B.seed_off = c->seed_off;
    B.pos_off = c->pos_off;
    B.seeds = c->seeds;
    B.seed_pos = c->seed_pos;
    B.pos = c->pos;
    B.pmap = c->pmap;
    B.seed_cap = n_seeds + 1;
    B.pos_cap = n_pos + 1;
    if (fetch) {
        RC(grow_host(c->h_seed_off, c->cap_h_so, nr1));
        RC(grow_host(c->h_pos_off, c->cap_h_po, nr1));
        RC(grow_host(c->h_seeds, c->cap_h_seeds, n_seeds + 1));
        RC(grow_host(c->h_pos, c->cap_h_pos, n_pos + 1));
    }
    if (co) {
        uint64_t ws = co->base_s + n_seeds + 1, wp = co->base_p + n_pos + 1;
        if (co->base_s == 0 && co->base_p == 0) {
            ws = (uint64_t)((double)ws * co->scale * 1.1);
            wp = (uint64_t)((double)wp * co->scale * 1.1);
        }
        RC(grow_host_keep(c->h_seeds, c->cap_h_seeds, ws, co->base_s, c->st_copy));
        RC(grow_host_keep(c->h_pos, c->cap_h_pos, wp, co->base_p, c->st_copy));
    }
    RC(gs_launch_finalize_emit(I, B, st));
    if (fetch) {
        /* seeds and per-read offsets are final here: copy them out on the
         * side stream while the positions are located */
        GS_CUDA(cudaEventRecord(c->ev_emit, st));
        GS_CUDA(cudaStreamWaitEvent(c->st_copy, c->ev_emit, 0));
        GS_CUDA(cudaMemcpyAsync(c->h_seed_off, c->seed_off, nr1 * 8, cudaMemcpyDeviceToHost,
                                c->st_copy));
        GS_CUDA(cudaMemcpyAsync(c->h_pos_off, c->pos_off, nr1 * 8, cudaMemcpyDeviceToHost,
                                c->st_copy));
        if (n_seeds)
            GS_CUDA(cudaMemcpyAsync(c->h_seeds, c->seeds, n_seeds * sizeof(gs_seed_rec),
                                    cudaMemcpyDeviceToHost, c->st_copy));
    }
    RC(gs_launch_locate(I, B, n_seeds, n_pos, st));
    if (co && n_reads) {
        gs_add_base_kernel<<<152 * 4, 256, 0, st>>>(c->seed_off, c->pos_off, n_reads, co->base_s,
                                                    co->base_p);
        GS_CUDA(cudaGetLastError());
    }
    GS_CUDA(cudaEventRecord(c->ev1, st));
    RC(fetch_small(&c->h_small[5], c->queue + 1, 4, st));
    RC(fetch_small(&c->h_small[10], c->queue + 2, 4, st));
    RC(fetch_small(&c->h_small[11], c->queue + 4, 4, st));
    if (B.work) RC(fetch_small(&c->h_small[6], c->d_work, 32, st));
    if (B.work) RC(fetch_small(&c->h_small[16], c->d_work + 4, 56, st));
    if (co) {
        /* after the small reads above: one copy engine serves both streams,
         * and this chunk's end should not wait for its own copy-out */
        GS_CUDA(cudaEventRecord(c->ev_done, st));
        GS_CUDA(cudaStreamWaitEvent(c->st_copy, c->ev_done, 0));
        GS_CUDA(cudaMemcpyAsync(c->h_seed_off + co->first_read, c->seed_off, (size_t)n_reads * 8,
                                cudaMemcpyDeviceToHost, c->st_copy));
        GS_CUDA(cudaMemcpyAsync(c->h_pos_off + co->first_read, c->pos_off, (size_t)n_reads * 8,
                                cudaMemcpyDeviceToHost, c->st_copy));
        if (n_seeds)
            GS_CUDA(cudaMemcpyAsync(c->h_seeds + co->base_s, c->seeds,
                                    n_seeds * sizeof(gs_seed_rec), cudaMemcpyDeviceToHost,
                                    c->st_copy));
        if (n_pos)
            GS_CUDA(cudaMemcpyAsync(c->h_pos + co->base_p, c->pos, n_pos * 4,
                                    cudaMemcpyDeviceToHost, c->st_copy));
        GS_CUDA(cudaEventRecord(c->ev_d2h, c->st_copy));
        co->n_seeds = n_seeds;
        co->n_pos = n_pos;
    }
    c->n_seeds = n_seeds;
    c->n_pos = n_pos;
    if (fetch && n_pos)
        GS_CUDA(cudaMemcpyAsync(c->h_pos, c->pos, n_pos * 4, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    if (fetch) GS_CUDA(cudaStreamSynchronize(c->st_copy));
    uint32_t flags = (uint32_t)(c->h_small[5] & 0xffffffffu);
    c->last_walkers = c->last_walker_cap ? (c->h_small[10] & 0xffffffffu) : 0;
    c->last_text_jobs = c->last_text_cap ? (c->h_small[11] & 0xffffffffu) : 0;
    if (!p->walker_slots && c->last_walker_cap && c->last_walkers >= c->last_walker_cap &&
        c->walker_per16 < 512u) {
        c->walker_per16 += c->walker_per16 / 2;
        if (c->walker_per16 > 512u) c->walker_per16 = 512u;
    }
    if (B.work) memcpy(c->work, &c->h_small[6], sizeof(c->work));
    if (B.work) memcpy(c->walk_counts, &c->h_small[16], sizeof(c->walk_counts));
    cudaEventElapsedTime(&c->t_search, c->ev_s0, c->ev_s1);
    cudaEventElapsedTime(&c->t_total, c->ev0, c->ev1);
    if (flags & GS_FLAG_WALK) {
        gs_set_error("sampled-SA walk exceeded seq_len+2 steps: index inconsistent");
        return GS_EWALK;
    }
    c->have_dev = 1;
    c->have_host = fetch;
    return GS_OK;
}

/* device -> host copy of the last pass's result (sizes known) */
static int fetch_result(gs_ctx *c)
{
    cudaStream_t st = c->st;
    size_t nr1 = (size_t)c->n_reads + 1;
    RC(grow_host(c->h_seed_off, c->cap_h_so, nr1));
    RC(grow_host(c->h_pos_off, c->cap_h_po, nr1));
    RC(grow_host(c->h_seeds, c->cap_h_seeds, c->n_seeds + 1));
    RC(grow_host(c->h_pos, c->cap_h_pos, c->n_pos + 1));
    GS_CUDA(cudaMemcpyAsync(c->h_seed_off, c->seed_off, nr1 * 8, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaMemcpyAsync(c->h_pos_off, c->pos_off, nr1 * 8, cudaMemcpyDeviceToHost, st));
    if (c->n_seeds)
        GS_CUDA(cudaMemcpyAsync(c->h_seeds, c->seeds, c->n_seeds * sizeof(gs_seed_rec),
                                cudaMemcpyDeviceToHost, st));
    if (c->n_pos)
        GS_CUDA(cudaMemcpyAsync(c->h_pos, c->pos, c->n_pos * 4, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    c->have_host = 1;
    return GS_OK;
}

/* Enqueues a whole pass with no host synchronisation: sizes come from the
 * device (work items, seed and position totals) and every buffer is bounded
 * by the capacities the context holds; overflow sets a flag. */
static int enqueue_pass(gs_ctx *c, const char *d_seqs, const uint64_t *d_offsets,
                        const uint32_t *d_lengths, uint32_t n_reads, const gs_params *p)
{
    const GsDevIndex &I = *gs_index_dev(c->idx);
    cudaStream_t st = c->st;
    size_t nr1 = (size_t)n_reads + 1;
    GsBatch B;
    memset(&B, 0, sizeof(B));
    B.seqs = d_seqs;
    B.offsets = d_offsets;
    B.lengths = d_lengths;
    B.n_reads = n_reads;
    B.k = p->k;
    B.smem = p->smem ? 1 : 0;
    B.n_mode = p->n_mode;
    B.lf_mode = p->lf_mode;
    B.max_occ = p->max_occ > 0 ? (uint32_t)p->max_occ : 0u;
    B.mem_next = p->mem_next;
    B.queue = c->queue;
    GS_CUDA(cudaMemsetAsync(c->queue, 0, 32, st));
    B.slot_off = c->slot_cnt;
    B.item_off = c->item_cnt;
    RC(gs_launch_prepare(I, B, GS_KERNEL_BATCHED, st));
    RC(exclusive_scan(c, c->slot_cnt, c->slot_off, nr1));
    RC(exclusive_scan(c, c->item_cnt, c->item_off, nr1));
    B.slot_off = c->slot_off;
    B.item_off = c->item_off;
    B.slots = c->slots;
    B.slot_cap = c->cap_slots;
    B.recmask = c->recmask;
    GS_CUDA(cudaMemsetAsync(c->recmask, 0, ((c->cap_slots + 31) / 32 + 1) * sizeof(uint32_t), st));
    B.item_cap = c->g_items;
    /* the walker buffer as the sizing pass left it; walkers beyond it are
     * left to the leftover pass */
    if (c->last_walker_cap && c->walkers) {
        B.walkers = c->walkers;
        B.walker_cap = c->last_walker_cap;
        if (c->last_text_cap && c->text_jobs && I.text_min) {
            B.text_jobs = c->text_jobs;
            B.text_cap = c->last_text_cap;
        }
    }
    RC(gs_launch_search(I, B, GS_KERNEL_BATCHED, p->queue_chunk, p->ctas_per_sm, 0, st));
    B.rd_nf = c->rd_nf;
    B.rd_nr = c->rd_nr;
    B.rd_nseeds = c->rd_nseeds;
    B.rd_npos = c->rd_npos;
    GS_CUDA(cudaMemsetAsync(c->rd_nseeds + n_reads, 0, 8, st));
    GS_CUDA(cudaMemsetAsync(c->rd_npos + n_reads, 0, 8, st));
    RC(gs_launch_finalize_count(I, B, st));
    RC(exclusive_scan(c, c->rd_nseeds, c->seed_off, nr1));
    RC(exclusive_scan(c, c->rd_npos, c->pos_off, nr1));
    B.seed_off = c->seed_off;
    B.pos_off = c->pos_off;
    B.seeds = c->seeds;
    B.seed_pos = c->seed_pos;
    B.pos = c->pos;
    B.pmap = c->pmap;
    B.seed_cap = c->cap_seeds < c->cap_seed_pos ? c->cap_seeds : c->cap_seed_pos;
    B.pos_cap = c->cap_pos < c->cap_pmap ? c->cap_pos : c->cap_pmap;
    RC(gs_launch_finalize_emit(I, B, st));
    RC(gs_launch_locate(I, B, 0, 0, st));
    return GS_OK;
}

static bool same_graph(const gs_ctx *c, const char *s, const uint64_t *o, const uint32_t *l,
                       uint32_t n, const gs_params *p)
{
    return c->gexec && c->g_seqs == s && c->g_offs == o && c->g_lens == l && c->g_n == n &&
           c->g_gen == gs_index_generation(c->idx) &&
           memcmp(&c->g_params, p, sizeof(gs_params)) == 0;
}

static int run_graph(gs_ctx *c, const char *d_seqs, const uint64_t *d_offsets,
                     const uint32_t *d_lengths, uint32_t n_reads, const gs_params *p, int fetch)
{
    cudaStream_t st = c->st;
    if (same_graph(c, d_seqs, d_offsets, d_lengths, n_reads, p)) {
        c->have_host = c->have_dev = 0;
        GS_CUDA(cudaEventRecord(c->ev0, st));
        GS_CUDA(cudaGraphLaunch(c->gexec, st));
        GS_CUDA(cudaEventRecord(c->ev1, st));
        GS_CUDA(cudaMemcpyAsync(&c->h_small[5], c->queue + 1, 4, cudaMemcpyDeviceToHost, st));
        GS_CUDA(cudaMemcpyAsync(&c->h_small[3], c->seed_off + n_reads, 8, cudaMemcpyDeviceToHost, st));
        GS_CUDA(cudaMemcpyAsync(&c->h_small[4], c->pos_off + n_reads, 8, cudaMemcpyDeviceToHost, st));
        GS_CUDA(cudaStreamSynchronize(st));
        uint32_t flags = (uint32_t)(c->h_small[5] & 0xffffffffu);
        uint64_t ns = c->h_small[3], np = c->h_small[4];
        bool fits = !(flags & GS_FLAG_OVERFLOW) && ns <= c->cap_seeds && ns <= c->cap_seed_pos &&
                    np <= c->cap_pos && np <= c->cap_pmap;
        if (fits) {
            if (flags & GS_FLAG_WALK) {
                gs_set_error("sampled-SA walk exceeded seq_len+2 steps: index inconsistent");
                return GS_EWALK;
            }
            c->n_reads = n_reads;
            c->n_seeds = ns;
            c->n_pos = np;
            c->have_dev = 1;
            cudaEventElapsedTime(&c->t_total, c->ev0, c->ev1);
            c->t_search = c->t_total;
            if (fetch) RC(fetch_result(c));
            return GS_OK;
        }
        /* outgrew the captured pass: size again below */
    }
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = NULL;
    }
    RC(run_pipeline(c, d_seqs, d_offsets, d_lengths, n_reads, p, fetch));
    if (!c->slots || !c->seeds || !c->pos || !c->seed_pos || !c->pmap) return GS_OK;
    /* capture a pass with the capacities this one needed */
    c->g_items = (uint32_t)(c->h_small[1] & 0xffffffffu);
    cudaGraph_t g = NULL;
    GS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_pass(c, d_seqs, d_offsets, d_lengths, n_reads, p);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return gs_cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->gexec = NULL;
        return gs_cuda_fail(e, "cudaGraphInstantiate");
    }
    c->g_seqs = d_seqs;
    c->g_offs = d_offsets;
    c->g_lens = d_lengths;
    c->g_n = n_reads;
    c->g_gen = gs_index_generation(c->idx);
    c->g_params = *p;
    return GS_OK;
}

extern "C" int gs_seed_device(gs_ctx *c, const char *d_seqs, const uint64_t *d_offsets,
                              const uint32_t *d_lengths, uint32_t n_reads, const gs_params *p,
                              int fetch_to_host)
{
    if (!c || (n_reads && (!d_seqs || !d_offsets || !d_lengths))) {
        gs_set_error("gs_seed_device: null argument");
        return GS_EINVAL;
    }
    RC(check_params(p));
    GS_ON_DEVICE(gs_index_device(c->idx));
    if (p->graph && p->kernel == GS_KERNEL_BATCHED && !p->count_work && n_reads)
        return run_graph(c, d_seqs, d_offsets, d_lengths, n_reads, p, fetch_to_host);
    return run_pipeline(c, d_seqs, d_offsets, d_lengths, n_reads, p, fetch_to_host);
}

/* A large batch whose reads lie in order in `seqs` runs as chunks of reads:
 * the reads go up on st_h2d chunk by chunk, each chunk is one pass on st,
 * and its results come down on st_copy while the next chunk searches.  The
 * host result is the batch's, as one pass would give it; the device keeps
 * only the last chunk's, so gs_result_device and the GPU text writer do
 * not apply (gs_result_write_text falls back to the host writer). */
static int seed_chunked(gs_ctx *c, const char *seqs, const uint64_t *offsets, uint32_t n_reads,
                        const gs_params *p, uint64_t bytes)
{
    /* the first and the last chunk are small: the first one's copy-in and
     * the last one's copy-out are the only copies nothing overlaps, and
     * every chunk costs its pass's fixed part (host syncs, kernel tails) */
    uint32_t K = (n_reads + GS_SEED_CHUNK_READS - 1) / GS_SEED_CHUNK_READS + 1;
    if (K > GS_SEED_MAX_CHUNKS) K = GS_SEED_MAX_CHUNKS;
    uint32_t first[GS_SEED_MAX_CHUNKS + 1];
    const double m = (double)n_reads / ((double)K - 2.0 + 2.0 * GS_SEED_END_FRACTION);
    first[0] = 0;
    for (uint32_t j = 1; j < K; j++)
        first[j] = (uint32_t)(GS_SEED_END_FRACTION * m + (double)(j - 1) * m);
    first[K] = n_reads;
    uint32_t max_n = 0;
    for (uint32_t j = 0; j < K; j++)
        if (first[j + 1] - first[j] > max_n) max_n = first[j + 1] - first[j];
    /* per-read arrays the copy-out reads, sized once for every chunk */
    RC(grow(c->seed_off, c->cap_so, (size_t)max_n + 1, c->st));
    RC(grow(c->pos_off, c->cap_po, (size_t)max_n + 1, c->st));
    RC(grow(c->d_seqs, c->cap_seqs, bytes + 1, c->st));
    GS_CUDA(cudaEventRecord(c->ev_done, c->st));
    GS_CUDA(cudaStreamWaitEvent(c->st_h2d, c->ev_done, 0));
    for (uint32_t j = 0; j < K; j++) {
        const uint64_t lo = offsets[first[j]];
        const uint64_t hi = j + 1 < K ? offsets[first[j + 1]] : bytes;
        if (hi > lo)
            GS_CUDA(cudaMemcpyAsync(c->d_seqs + lo, seqs + lo, hi - lo, cudaMemcpyHostToDevice,
                                    c->st_h2d));
        GS_CUDA(cudaEventRecord(c->ev_h2d[j], c->st_h2d));
    }
    RC(grow_host(c->h_seed_off, c->cap_h_so, (size_t)n_reads + 1));
    RC(grow_host(c->h_pos_off, c->cap_h_po, (size_t)n_reads + 1));
    uint64_t bs = 0, bp = 0, walkers = 0, text_jobs = 0, work[4] = {0, 0, 0, 0};
    float t_search = 0.f, t_total = 0.f;
    int rc = GS_OK;
    for (uint32_t j = 0; j < K && rc == GS_OK; j++) {
        const uint32_t nj = first[j + 1] - first[j];
        const cudaError_t e = cudaStreamWaitEvent(c->st, c->ev_h2d[j], 0);
        if (e != cudaSuccess) {
            rc = gs_cuda_fail(e, "cudaStreamWaitEvent(chunk)");
            break;
        }
        GsChunkOut co;
        memset(&co, 0, sizeof(co));
        co.first_read = first[j];
        co.base_s = bs;
        co.base_p = bp;
        co.scale = (double)n_reads / (double)(nj ? nj : 1);
        co.wait_d2h = j > 0;
        rc = run_pipeline(c, c->d_seqs, c->d_offsets + first[j], c->d_lengths + first[j], nj, p,
                          0, &co);
        if (rc) break;
        bs += co.n_seeds;
        bp += co.n_pos;
        walkers += c->last_walkers;
        text_jobs += c->last_text_jobs;
        for (int w = 0; w < 4; w++) work[w] += c->work[w];
        t_search += c->t_search;
        t_total += c->t_total;
    }
    /* no copy may outlive the call: the caller owns the host buffers */
    cudaStreamSynchronize(c->st_h2d);
    cudaStreamSynchronize(c->st_copy);
    cudaStreamSynchronize(c->st);
    c->have_dev = 0;
    if (rc) {
        c->have_host = 0;
        return rc;
    }
    c->h_seed_off[n_reads] = bs;
    c->h_pos_off[n_reads] = bp;
    c->n_reads = n_reads;
    c->n_seeds = bs;
    c->n_pos = bp;
    c->last_walkers = walkers;
    c->last_text_jobs = text_jobs;
    memcpy(c->work, work, sizeof(work));
    c->t_search = t_search;
    c->t_total = t_total;
    c->have_host = 1;
    return GS_OK;
}

extern "C" int gs_seed(gs_ctx *c, const char *seqs, const uint64_t *offsets,
                       const uint32_t *lengths, uint32_t n_reads, const gs_params *p)
{
    if (!c || (n_reads && (!seqs || !offsets || !lengths))) {
        gs_set_error("gs_seed: null argument");
        return GS_EINVAL;
    }
    RC(check_params(p));
    GS_ON_DEVICE(gs_index_device(c->idx));
    /* offsets and lengths first; the end of the last base comes from a
     * reduction on the device, then the bases themselves */
    RC(grow(c->d_offsets, c->cap_offsets, (size_t)n_reads + 1, c->st));
    RC(grow(c->d_lengths, c->cap_lengths, (size_t)n_reads + 1, c->st));
    uint64_t bytes = 0;
    if (n_reads) {
        GS_CUDA(cudaMemcpyAsync(c->d_offsets, offsets, (size_t)n_reads * 8, cudaMemcpyHostToDevice,
                                c->st));
        GS_CUDA(cudaMemcpyAsync(c->d_lengths, lengths, (size_t)n_reads * 4, cudaMemcpyHostToDevice,
                                c->st));
        GS_CUDA(cudaMemsetAsync(c->d_max, 0, 16, c->st));
        gs_max_end_kernel<<<(n_reads + 255) / 256, 256, 0, c->st>>>(
            c->d_offsets, c->d_lengths, n_reads, (unsigned long long *)c->d_max);
        GS_CUDA(cudaGetLastError());
        RC(fetch_small(&c->h_small[12], c->d_max, 16, c->st));
        GS_CUDA(cudaStreamSynchronize(c->st));
        bytes = c->h_small[12];
        /* chunks would cut the reference's cross-read neighbour scan */
        const bool cross = !p->smem && p->mem_next == GS_MEM_NEXT_GPUSEED;
        if (n_reads >= GS_SEED_CHUNK_READS && c->h_small[13] == 0 && !cross)
            return seed_chunked(c, seqs, offsets, n_reads, p, bytes);
    }
    RC(grow(c->d_seqs, c->cap_seqs, bytes + 1, c->st));
    if (bytes) GS_CUDA(cudaMemcpyAsync(c->d_seqs, seqs, bytes, cudaMemcpyHostToDevice, c->st));
    return run_pipeline(c, c->d_seqs, c->d_offsets, c->d_lengths, n_reads, p, 1);
}

extern "C" int gs_result_host(gs_ctx *c, gs_result_view *out)
{
    if (!c || !out) return GS_EINVAL;
    if (!c->have_host) {
        gs_set_error("no host result: last call failed or left it on the device");
        return GS_ESTATE;
    }
    out->n_reads = c->n_reads;
    out->n_seeds = c->n_seeds;
    out->n_pos = c->n_pos;
    out->read_seed_off = c->h_seed_off;
    out->read_pos_off = c->h_pos_off;
    out->seeds = c->h_seeds;
    out->pos = c->h_pos;
    return GS_OK;
}

extern "C" int gs_result_device(gs_ctx *c, gs_result_view *out)
{
    if (!c || !out) return GS_EINVAL;
    if (!c->have_dev) {
        gs_set_error("no device result");
        return GS_ESTATE;
    }
    out->n_reads = c->n_reads;
    out->n_seeds = c->n_seeds;
    out->n_pos = c->n_pos;
    out->read_seed_off = c->seed_off;
    out->read_pos_off = c->pos_off;
    out->seeds = c->seeds;
    out->pos = c->pos;
    return GS_OK;
}

/* ------------------------------------------------------------------ */
/* text records (seed_gen.cu:3625-3647) */

struct OutBuf {
    int fd;
    char *b;
    size_t n, cap;
    int err;
};

static void ob_flush(OutBuf *o)
{
    size_t off = 0;
    while (off < o->n && !o->err) {
        ssize_t w = write(o->fd, o->b + off, o->n - off);
        if (w < 0) {
            if (errno == EINTR) continue;
            o->err = 1;
            break;
        }
        off += (size_t)w;
    }
    o->n = 0;
}

static inline void ob_put(OutBuf *o, const char *s, size_t n)
{
    if (o->n + n > o->cap) ob_flush(o);
    memcpy(o->b + o->n, s, n);
    o->n += n;
}

static inline void ob_u32(OutBuf *o, uint32_t v)
{
    char t[12];
    int i = 12;
    do {
        t[--i] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    ob_put(o, t + i, (size_t)(12 - i));
}

extern "C" int gs_result_write_text_host(gs_ctx *c, int fd, uint32_t first_read_no, int smem)
{
    if (!c) return GS_EINVAL;
    if (!c->have_host) {
        gs_set_error("no host result to print");
        return GS_ESTATE;
    }
    OutBuf o = {fd, (char *)malloc(1 << 20), 0, 1 << 20, 0};
    if (!o.b) return GS_ENOMEM;
    static const char h0[] = "/*===================================";
    static const char h1[] = " seeds in read no. ";
    static const char h2[] = " (Read[begin, End] -> starting position(s) on the reference)"
                             "===================================*/\n";
    for (uint32_t r = 0; r < c->n_reads; r++) {
        ob_put(&o, h0, sizeof(h0) - 1);
        if (smem) ob_put(&o, "SMEM", 4);
        else ob_put(&o, "MEM", 3);
        ob_put(&o, h1, sizeof(h1) - 1);
        ob_u32(&o, first_read_no + r);
        ob_put(&o, h2, sizeof(h2) - 1);
        const uint32_t *pos = c->h_pos + c->h_pos_off[r];
        for (uint64_t s = c->h_seed_off[r]; s < c->h_seed_off[r + 1]; s++) {
            const gs_seed_rec &S = c->h_seeds[s];
            char sg = ((uint32_t)S.y >> 31) ? '-' : '+';
            for (uint32_t q = 0; q < S.n_pos; q++, pos++) {
                if (q == 0) {
                    ob_put(&o, "\nRead[", 6);
                    ob_u32(&o, (uint32_t)S.x & 0x7fffffffu);
                    ob_put(&o, ", ", 2);
                    ob_u32(&o, (uint32_t)S.y & 0x7fffffffu);
                    ob_put(&o, "] -> ", 5);
                } else {
                    ob_put(&o, ", ", 2);
                }
                ob_put(&o, &sg, 1);
                ob_u32(&o, *pos);
            }
        }
        ob_put(&o, "\n", 1);
    }
    ob_flush(&o);
    free(o.b);
    if (o.err) {
        gs_set_error("write failed");
        return GS_EIO;
    }
    return GS_OK;
}

/* Text records formatted on the GPU from the device result (gs_text.cu):
 * token lengths, one in-place scan to byte offsets, the bytes. */
static int format_text_device(gs_ctx *c, uint32_t first_read_no, int smem, uint64_t *n_bytes)
{
    if (!c->have_dev) {
        gs_set_error("no device result to print");
        return GS_ESTATE;
    }
    cudaStream_t st = c->st;
    const uint64_t n_tok = 2ull * c->n_reads + c->n_seeds + c->n_pos;
    RC(grow(c->t_sread, c->cap_t_sread, (size_t)c->n_seeds + 1, c->st));
    RC(grow(c->t_off, c->cap_t_off, (size_t)n_tok + 1, c->st));
    GsTextArgs a;
    memset(&a, 0, sizeof(a));
    a.n_reads = c->n_reads;
    a.n_seeds = c->n_seeds;
    a.n_pos = c->n_pos;
    a.seed_off = c->seed_off;
    a.pos_off = c->pos_off;
    a.seeds = c->seeds;
    a.seed_pos = c->seed_pos;
    a.pmap = c->pmap;
    a.pos = c->pos;
    a.first_read_no = first_read_no;
    a.smem = smem ? 1 : 0;
    a.sread = c->t_sread;
    a.off = c->t_off;
    GS_CUDA(cudaMemsetAsync(c->t_off + n_tok, 0, 8, st));
    RC(gs_launch_text_lengths(a, st));
    RC(exclusive_scan(c, c->t_off, c->t_off, (size_t)n_tok + 1));
    GS_CUDA(cudaMemcpyAsync(&c->h_small[11], c->t_off + n_tok, 8, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    const uint64_t total = c->h_small[11];
    RC(grow(c->t_text, c->cap_t_text, (size_t)total + 1, c->st));
    a.text = c->t_text;
    RC(gs_launch_text_write(a, st));
    *n_bytes = total;
    return GS_OK;
}

extern "C" int gs_result_text_device(gs_ctx *c, uint32_t first_read_no, int smem,
                                     const char **d_text, uint64_t *n_bytes)
{
    if (!c || !d_text || !n_bytes) return GS_EINVAL;
    uint64_t n = 0;
    RC(format_text_device(c, first_read_no, smem, &n));
    GS_CUDA(cudaStreamSynchronize(c->st));
    *d_text = c->t_text;
    *n_bytes = n;
    return GS_OK;
}

static int write_all(int fd, const char *b, size_t n)
{
    size_t off = 0;
    while (off < n) {
        ssize_t w = write(fd, b + off, n - off);
        if (w < 0) {
            if (errno == EINTR) continue;
            gs_set_error("write failed: %s", strerror(errno));
            return GS_EIO;
        }
        off += (size_t)w;
    }
    return GS_OK;
}

#define GS_TEXT_CHUNK ((size_t)64 << 20)

/* The -o records: formatted on the GPU when the device result is there,
 * copied out in 64 MiB chunks through two pinned buffers (the next chunk's
 * copy overlaps the write of the last); otherwise by the host writer. */
extern "C" int gs_result_write_text(gs_ctx *c, int fd, uint32_t first_read_no, int smem)
{
    if (!c) return GS_EINVAL;
    if (!c->have_dev) return gs_result_write_text_host(c, fd, first_read_no, smem);
    uint64_t total = 0;
    RC(format_text_device(c, first_read_no, smem, &total));
    for (int i = 0; i < 2; i++) {
        if (!c->h_text[i]) GS_CUDA(cudaMallocHost(&c->h_text[i], GS_TEXT_CHUNK));
        if (!c->t_ev[i]) GS_CUDA(cudaEventCreateWithFlags(&c->t_ev[i], cudaEventDisableTiming));
    }
    cudaStream_t st = c->st;
    uint64_t done = 0;
    int i = 0;
    if (total) {
        GS_CUDA(cudaMemcpyAsync(c->h_text[0], c->t_text, (size_t)(total < GS_TEXT_CHUNK ? total : GS_TEXT_CHUNK),
                                cudaMemcpyDeviceToHost, st));
        GS_CUDA(cudaEventRecord(c->t_ev[0], st));
    }
    while (done < total) {
        const size_t n = (size_t)(total - done < GS_TEXT_CHUNK ? total - done : GS_TEXT_CHUNK);
        const uint64_t next = done + n;
        if (next < total) {
            const size_t m = (size_t)(total - next < GS_TEXT_CHUNK ? total - next : GS_TEXT_CHUNK);
            GS_CUDA(cudaMemcpyAsync(c->h_text[(i + 1) & 1], c->t_text + next, m,
                                    cudaMemcpyDeviceToHost, st));
            GS_CUDA(cudaEventRecord(c->t_ev[(i + 1) & 1], st));
        }
        GS_CUDA(cudaEventSynchronize(c->t_ev[i & 1]));
        int rc = write_all(fd, c->h_text[i & 1], n);
        if (rc) {
            cudaStreamSynchronize(st);
            return rc;
        }
        done = next;
        i++;
    }
    return GS_OK;
}

/* ------------------------------------------------------------------ */
/* autotuner: coordinate descent over the batched search's launch knobs,
 * each setting timed (search kernels only, CUDA events) on the first
 * `sample` reads; the fastest setting is written back into *p. */

extern "C" int gs_autotune(gs_ctx *c, const char *d_seqs, const uint64_t *d_offsets,
                           const uint32_t *d_lengths, uint32_t n_reads, gs_params *p,
                           uint32_t sample, float *best_ms)
{
    if (!c || !p || (n_reads && (!d_seqs || !d_offsets || !d_lengths))) {
        gs_set_error("gs_autotune: null argument");
        return GS_EINVAL;
    }
    RC(check_params(p));
    GS_ON_DEVICE(gs_index_device(c->idx));
    uint32_t n = sample && sample < n_reads ? sample : n_reads;
    auto eval = [&](const gs_params &q, float &ms) -> int {
        float best = 1e30f;
        for (int rep = 0; rep < 2; rep++) {
            int rc = run_pipeline(c, d_seqs, d_offsets, d_lengths, n, &q, 0);
            if (rc) return rc;
            if (rep > 0 || n < 1000) best = c->t_search < best ? c->t_search : best;
        }
        ms = best;
        return GS_OK;
    };
    gs_params best = *p;
    /* the batched search has two knobs (start-pass queue grab, CTAs per
     * SM); the lockstep form also its two hand-over thresholds */
    const bool lock = p->kernel == GS_KERNEL_LOCKSTEP;
    best.kernel = lock ? GS_KERNEL_LOCKSTEP : GS_KERNEL_BATCHED;
    best.count_work = 0;
    if (!best.queue_chunk) best.queue_chunk = GS_QUEUE_CHUNK;
    if (!best.handoff_lanes) best.handoff_lanes = GS_HANDOFF_LANES;
    if (!best.handoff_steps) best.handoff_steps = GS_HANDOFF_STEPS;
    float bt = 0;
    RC(eval(best, bt));
    static const int qcs[] = {1, 2, 4, 8, 16};
    static const int lanes[] = {-1, 1, 2, 3, 4, 6, 8};
    static const int steps[] = {2, 3, 4, 6, 8, 12};
    static const int ctas[] = {0, 2, 3, 4};
    for (int round = 0; round < 2; round++) {
        for (int dim = 0; dim < 4; dim++) {
            if (!lock && (dim == 1 || dim == 2)) continue;
            const int *vals = dim == 0 ? qcs : dim == 1 ? lanes : dim == 2 ? steps : ctas;
            int nv = dim == 0 ? 5 : dim == 1 ? 7 : dim == 2 ? 6 : 4;
            for (int i = 0; i < nv; i++) {
                gs_params q = best;
                int *f = dim == 0 ? &q.queue_chunk : dim == 1 ? &q.handoff_lanes
                         : dim == 2 ? &q.handoff_steps : &q.ctas_per_sm;
                if (*f == vals[i]) continue;
                *f = vals[i];
                float t = 0;
                RC(eval(q, t));
                if (t < bt * 0.99f) {
                    bt = t;
                    best = q;
                }
            }
        }
    }
    best.kernel = p->kernel;
    best.count_work = p->count_work;
    *p = best;
    if (best_ms) *best_ms = bt;
    return GS_OK;
}
