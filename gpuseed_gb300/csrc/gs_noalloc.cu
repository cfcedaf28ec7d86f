/*
 * gs_noalloc.cu -- the batched seeding pass without any allocation.
 *
 * For callers that must not allocate device memory while they run: a
 * serving process that reserved its HBM budget at start-up, or code that
 * cannot afford the device-wide synchronisation cudaMalloc/cudaFree imply
 * while other streams are busy.  gs_seed_device() grows a per-context
 * workspace with cudaMalloc; gs_seed_noalloc() instead keeps every scratch
 * buffer of the pass (candidate slots, per-read counters, work queue, scan
 * temporaries, the position-to-seed map) in one file-scope device array of
 * GS_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library holds
 * until the process exits.  The caller passes the reads and the output
 * buffers; results are written only there.
 *
 * The search is the lockstep form without the tail-pass hand-over
 * (GS_KERNEL_LOCKSTEP with handoff_lanes < 0): it needs neither the walker
 * buffer of the batched form nor the hand-over records, whose sizes follow
 * the batch.  Its seeds and positions are the same integers.
 *
 * Host code must not use the array's name as a device address: on the host
 * it names a shadow object.  The device address is taken once per device
 * with cudaGetSymbolAddress, with that device current, on the first call
 * made on that device -- make that first call before any stream capture.
 * The address is kept for the life of the process, so the device must not
 * be reset (cudaDeviceReset) between calls.  Each call synchronises its
 * stream three times, to size the pass from counts on the device.
 *
 * All calls share the one array and leave their data in it; each call
 * clears what has to start at zero.  Calls whose work overlaps on the GPU
 * (different streams, different host threads) race on the array: serialise
 * them.
 */
#include "gs_internal.h"

#include <cub/cub.cuh>

#include <mutex>
#include <string.h>

static __device__ __align__(256) unsigned char g_noalloc_scratch[GS_NOALLOC_SCRATCH_BYTES];

#define GS_NA_MAX_DEVICES 64
static void *g_scratch_dev[GS_NA_MAX_DEVICES];
static std::mutex g_scratch_mu;

const GsDevIndex *gs_index_dev(const gs_index *idx);
int gs_index_device(const gs_index *idx);

static int scratch_address(int dev, unsigned char **out)
{
    if (dev < 0 || dev >= GS_NA_MAX_DEVICES) {
        gs_set_error("gs_seed_noalloc: device %d outside [0, %d)", dev, GS_NA_MAX_DEVICES);
        return GS_EINVAL;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_dev[dev]) {
        void *p = NULL;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return gs_cuda_fail(e, "cudaGetSymbolAddress(scratch)");
        g_scratch_dev[dev] = p;
    }
    *out = (unsigned char *)g_scratch_dev[dev];
    return GS_OK;
}

/* bump allocator over the scratch array */
struct Carve {
    unsigned char *base;
    size_t used, cap;
    template <class T>
    T *take(size_t n)
    {
        size_t off = (used + 255) & ~(size_t)255;
        size_t bytes = n * sizeof(T);
        if (off + bytes > cap) return NULL;
        used = off + bytes;
        return (T *)(base + off);
    }
};

#define NA_RC(x)                 \
    do {                         \
        int _rc = (x);           \
        if (_rc) return _rc;     \
    } while (0)

extern "C" int gs_seed_noalloc(gs_index *idx, const char *d_seqs, const uint64_t *d_offsets,
                               const uint32_t *d_lengths, uint32_t n_reads, const gs_params *p,
                               void *cuda_stream, gs_seed_rec *d_seeds, uint64_t seed_cap,
                               uint32_t *d_pos, uint64_t pos_cap, uint64_t *d_read_seed_off,
                               uint64_t *d_read_pos_off, uint64_t *n_seeds_out,
                               uint64_t *n_pos_out)
{
    if (!idx || !p || !d_read_seed_off || !d_read_pos_off || !n_seeds_out || !n_pos_out ||
        (n_reads && (!d_seqs || !d_offsets || !d_lengths))) {
        gs_set_error("gs_seed_noalloc: null argument");
        return GS_EINVAL;
    }
    if (p->kernel != GS_KERNEL_BATCHED && p->kernel != GS_KERNEL_LOCKSTEP) {
        gs_set_error("gs_seed_noalloc: kernel must be GS_KERNEL_BATCHED or GS_KERNEL_LOCKSTEP "
                     "(both run the lockstep search here)");
        return GS_EINVAL;
    }
    if (p->k < GS_K0 || (p->n_mode != GS_N_WILDCARD && p->n_mode != GS_N_STOP) ||
        (p->lf_mode != GS_LF_GPUSEED && p->lf_mode != GS_LF_BWA) ||
        (p->mem_next != GS_MEM_NEXT_READ && p->mem_next != GS_MEM_NEXT_GPUSEED)) {
        gs_set_error("gs_seed_noalloc: k must be >= 13 and modes in range");
        return GS_EINVAL;
    }
    if (n_reads > GS_NOALLOC_MAX_READS) {
        gs_set_error("gs_seed_noalloc: %u reads, at most %u per call", n_reads,
                     (unsigned)GS_NOALLOC_MAX_READS);
        return GS_EINVAL;
    }
    const int dev = gs_index_device(idx);
    GS_ON_DEVICE(dev);
    unsigned char *scratch = NULL;
    NA_RC(scratch_address(dev, &scratch));
    cudaStream_t st = (cudaStream_t)cuda_stream;
    const GsDevIndex &I = *gs_index_dev(idx);
    const size_t nr1 = (size_t)n_reads + 1;

    Carve cv = {scratch, 0, GS_NOALLOC_SCRATCH_BYTES};
    uint64_t *slot_cnt = cv.take<uint64_t>(nr1), *slot_off = cv.take<uint64_t>(nr1);
    uint32_t *item_cnt = cv.take<uint32_t>(nr1), *item_off = cv.take<uint32_t>(nr1);
    uint32_t *rd_nf = cv.take<uint32_t>(nr1), *rd_nr = cv.take<uint32_t>(nr1);
    uint64_t *rd_nseeds = cv.take<uint64_t>(nr1), *rd_npos = cv.take<uint64_t>(nr1);
    uint32_t *queue = cv.take<uint32_t>(4);
    size_t cub_bytes = 0, b2 = 0;
    GS_CUDA(cub::DeviceScan::ExclusiveSum(NULL, cub_bytes, slot_cnt, slot_off, (int64_t)nr1, st));
    GS_CUDA(cub::DeviceScan::ExclusiveSum(NULL, b2, item_cnt, item_off, (int64_t)nr1, st));
    if (b2 > cub_bytes) cub_bytes = b2;
    unsigned char *cub_tmp = cv.take<unsigned char>(cub_bytes + 256);
    GsRec *slots = cv.take<GsRec>(GS_NOALLOC_MAX_SLOTS);
    uint32_t *recmask = cv.take<uint32_t>(GS_NOALLOC_MAX_SLOTS / 32 + 1);
    uint64_t *seed_pos = cv.take<uint64_t>(GS_NOALLOC_MAX_SEEDS);
    uint32_t *pmap = cv.take<uint32_t>(GS_NOALLOC_MAX_POS);
    if (!slot_cnt || !slot_off || !item_cnt || !item_off || !rd_nf || !rd_nr || !rd_nseeds ||
        !rd_npos || !queue || !cub_tmp || !slots || !recmask || !seed_pos || !pmap) {
        gs_set_error("gs_seed_noalloc: scratch layout exceeds %u bytes",
                     (unsigned)GS_NOALLOC_SCRATCH_BYTES);
        return GS_ENOMEM;
    }

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
    B.queue = queue;
    GS_CUDA(cudaMemsetAsync(queue, 0, 4 * sizeof(uint32_t), st));

    /* slots and work items per read */
    B.slot_off = slot_cnt;
    B.item_off = item_cnt;
    NA_RC(gs_launch_prepare(I, B, GS_KERNEL_LOCKSTEP, st));
    GS_CUDA(cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, slot_cnt, slot_off, (int64_t)nr1, st));
    GS_CUDA(cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, item_cnt, item_off, (int64_t)nr1, st));
    uint64_t n_slots = 0;
    uint32_t n_items = 0;
    GS_CUDA(cudaMemcpyAsync(&n_slots, slot_off + n_reads, 8, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaMemcpyAsync(&n_items, item_off + n_reads, 4, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    if (n_slots > GS_NOALLOC_MAX_SLOTS) {
        gs_set_error("gs_seed_noalloc: %llu candidate slots (2 per start position of k), at most %u "
                     "per call", (unsigned long long)n_slots, (unsigned)GS_NOALLOC_MAX_SLOTS);
        return GS_EINVAL;
    }
    B.slot_off = slot_off;
    B.item_off = item_off;
    B.slots = slots;
    B.slot_cap = GS_NOALLOC_MAX_SLOTS;
    B.recmask = recmask;
    GS_CUDA(cudaMemsetAsync(recmask, 0, ((n_slots + 31) / 32 + 1) * sizeof(uint32_t), st));
    B.item_cap = n_items;
    /* the lockstep form without hand-over (B.cont stays NULL): it needs no
     * walker buffer and no hand-over records; its launch knobs are its own
     * defaults, not the caller's, which are tuned for the batched form */
    NA_RC(gs_launch_search(I, B, GS_KERNEL_LOCKSTEP, 0, 0, n_items, st));

    /* filters and counts; offsets go straight to the caller's arrays */
    B.rd_nf = rd_nf;
    B.rd_nr = rd_nr;
    B.rd_nseeds = rd_nseeds;
    B.rd_npos = rd_npos;
    GS_CUDA(cudaMemsetAsync(rd_nseeds + n_reads, 0, 8, st));
    GS_CUDA(cudaMemsetAsync(rd_npos + n_reads, 0, 8, st));
    NA_RC(gs_launch_finalize_count(I, B, st));
    GS_CUDA(cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, rd_nseeds, d_read_seed_off,
                                          (int64_t)nr1, st));
    GS_CUDA(cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, rd_npos, d_read_pos_off, (int64_t)nr1,
                                          st));
    uint64_t n_seeds = 0, n_pos = 0;
    GS_CUDA(cudaMemcpyAsync(&n_seeds, d_read_seed_off + n_reads, 8, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaMemcpyAsync(&n_pos, d_read_pos_off + n_reads, 8, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    *n_seeds_out = n_seeds;
    *n_pos_out = n_pos;
    if (n_seeds > GS_NOALLOC_MAX_SEEDS || n_pos > GS_NOALLOC_MAX_POS) {
        gs_set_error("gs_seed_noalloc: %llu seeds / %llu positions, at most %u / %u per call",
                     (unsigned long long)n_seeds, (unsigned long long)n_pos,
                     (unsigned)GS_NOALLOC_MAX_SEEDS, (unsigned)GS_NOALLOC_MAX_POS);
        return GS_EOVERFLOW;
    }
    if (n_seeds > seed_cap || n_pos > pos_cap || (n_seeds && !d_seeds) || (n_pos && !d_pos)) {
        gs_set_error("gs_seed_noalloc: output needs %llu seeds and %llu positions, buffers hold "
                     "%llu and %llu", (unsigned long long)n_seeds, (unsigned long long)n_pos,
                     (unsigned long long)seed_cap, (unsigned long long)pos_cap);
        return GS_EOVERFLOW;
    }
    B.seed_off = d_read_seed_off;
    B.pos_off = d_read_pos_off;
    B.seeds = d_seeds;
    B.seed_pos = seed_pos;
    B.pos = d_pos;
    B.pmap = pmap;
    B.seed_cap = n_seeds;
    B.pos_cap = n_pos;
    NA_RC(gs_launch_finalize_emit(I, B, st));
    NA_RC(gs_launch_locate(I, B, n_seeds, n_pos, st));
    uint32_t flags = 0;
    GS_CUDA(cudaMemcpyAsync(&flags, queue + 1, 4, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    if (flags & GS_FLAG_WALK) {
        gs_set_error("sampled-SA walk exceeded seq_len+2 steps: index inconsistent");
        return GS_EWALK;
    }
    return GS_OK;
}
