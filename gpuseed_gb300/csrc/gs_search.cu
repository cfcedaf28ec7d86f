/*
 * gs_search.cu -- seed-interval search (the hot path).
 *
 * Semantics (restated from find_seed_intervals_gpu, seed_gen.cu:2087-2413):
 *   forward candidate e (end):   13-mer R[e-12..e] from the k-mer table, then
 *                                extend left while the interval stays valid;
 *                                record ([b, e+1), I) if e+1-b >= k;
 *   reverse candidate s (start): complement codes, 13-mer at s, extend right;
 *                                record ([s, x+1) | bit 31, I) if x+1-s >= k.
 * A candidate may stop early once its interval has the same size as that of
 * its neighbour toward the longer match (e+1 forward, s-1 reverse) at the
 * same far end: both filters drop such a record, so it need not be produced.
 * The reference prunes with 30 warp shuffles per step over uninitialised
 * flags (:2100-2204); this file uses a defined rule: compare with the nearest
 * still-extending lane to the right, from a GS_HIST-deep own history.
 *
 * Two launch forms:
 *   gs_search_batched: persistent CTAs; each warp takes work items
 *     (read, strand, 31 candidates + 1 helper lane) from a global queue and
 *     steps its 32 candidates in lockstep, one occ lookup per lane per step.
 *   gs_search_plain:   one thread per read, candidates one after another,
 *     containment history in a per-read global array.
 */
#include "gs_fm.cuh"



/* ------------------------------------------------------------------ */
/* 13-mer interval table (pre_calc_seed_intervals_gpu, seed_gen.cu:2648) */

__global__ void gs_kmer_kernel(GsDevIndex I, uint2 *table, uint32_t n)
{
    uint32_t patt = blockIdx.x * blockDim.x + threadIdx.x;
    if (patt >= n) return;
    uint32_t l = 0, u = I.seq_len;
    for (int i = 0; i < GS_K0; i++) {
        gs_step(I, l, u, (patt >> (i << 1)) & 3u);
        if (l > u) break;
    }
    table[patt] = make_uint2(l, u);
}

int gs_build_kmer_table(const GsDevIndex &I, uint2 *table, cudaStream_t st)
{
    uint32_t n = 1u << (2 * GS_K0);
    gs_kmer_kernel<<<(n + 255) / 256, 256, 0, st>>>(I, table, n);
    GS_CUDA(cudaGetLastError());
    return GS_OK;
}

/* Longer start table, built in three passes over all kx-mers (base j at
 * bits 2j, processed first, i.e. the string's last character sits at bits
 * 0-1):
 *   1. (l,u) from the 13-mer prefix interval plus kx-13 steps;
 *   2. the forced right extension of each kx-mer X: the base c with
 *      count(Xc) == count(X) > 0, if any.  Xc's interval is one step with X's
 *      first character from the kx-mer table entry of (X without its first
 *      character)·c;
 *   3. packing: entry.x = l, entry.y = size << 3 | code, code 0-3 the forced
 *      base, 4 none, 7 "size does not fit 29 bits: start from the 13-mer".
 * A candidate whose kx-mer is always followed by its neighbour's next base is
 * contained in that neighbour (see the file comment) and needs no walk;
 * gs_search_plain stops such candidates at their start. */
__global__ void gs_kmerx_kernel(GsDevIndex I, uint2 *table, int kx, uint64_t n)
{
    for (uint64_t patt = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; patt < n;
         patt += (uint64_t)gridDim.x * blockDim.x) {
        uint2 iv = __ldg(&I.kmer[patt & ((1u << (2 * GS_K0)) - 1u)]);
        uint32_t l = iv.x, u = iv.y;
        for (int i = GS_K0; i < kx && l <= u; i++) gs_step(I, l, u, (uint32_t)(patt >> (i << 1)) & 3u);
        table[patt] = make_uint2(l, u);
    }
}

__global__ void gs_kmerx_code_kernel(GsDevIndex I, const uint2 *table, int kx, uint64_t n,
                                     uint8_t *code)
{
    const uint64_t mask = n - 1;
    for (uint64_t X = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; X < n;
         X += (uint64_t)gridDim.x * blockDim.x) {
        uint2 e = table[X];
        uint8_t out = 4;
        if (e.x <= e.y) {
            uint32_t size = e.y - e.x + 1u;
            uint32_t first = (uint32_t)(X >> (2 * (kx - 1))) & 3u;   /* X's first character */
            for (uint32_t c = 0; c < 4; c++) {
                uint2 y = table[((X << 2) | c) & mask];
                if (y.x > y.y) continue;
                uint32_t l = y.x, u = y.y;
                gs_step(I, l, u, first);
                if (l <= u && u - l + 1u == size) {
                    out = (uint8_t)c;
                    break;
                }
            }
        }
        code[X] = out;
    }
}

__global__ void gs_kmerx_pack_kernel(uint2 *table, uint64_t n, const uint8_t *code)
{
    for (uint64_t X = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; X < n;
         X += (uint64_t)gridDim.x * blockDim.x) {
        uint2 e = table[X];
        uint32_t size = e.x <= e.y ? e.y - e.x + 1u : 0u;
        uint32_t c = code[X];
        if (size >= (1u << 29)) {
            size = 0;
            c = 7;
        }
        table[X] = make_uint2(e.x, (size << 3) | c);
    }
}

int gs_build_kmerx_table(const GsDevIndex &I, uint2 *table, int kx, cudaStream_t st)
{
    uint64_t n = 1ull << (2 * kx);
    gs_kmerx_kernel<<<152 * 64, 256, 0, st>>>(I, table, kx, n);
    GS_CUDA(cudaGetLastError());
    uint8_t *code = NULL;
    GS_CUDA(cudaMallocAsync(&code, n, st));
    gs_kmerx_code_kernel<<<152 * 64, 256, 0, st>>>(I, table, kx, n, code);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        gs_kmerx_pack_kernel<<<152 * 64, 256, 0, st>>>(table, n, code);
        e = cudaGetLastError();
    }
    cudaFreeAsync(code, st);
    if (e != cudaSuccess) return gs_cuda_fail(e, "k-mer start table");
    return GS_OK;
}

/* Start of a candidate: the interval of its first KT bases (forward: the
 * bases anchor, anchor-1, ...; reverse: the complement codes anchor,
 * anchor+1, ...; the first base at bits 0-1).  Returns false when one of the
 * first 13 bases is not ACGT (no search, seed_gen.cu:2132-2143).  A non-ACGT
 * base at positions 13..KT-1 takes the 13-mer start and steps over it like
 * the main loop does.  pos = far end reached; alive = interval non-empty;
 * contained (FORCED only) = the start string is always followed by the
 * neighbour's next base (the candidate needs no walk and produces no record). */
template <int NSTOP, bool FORCED>
__device__ __forceinline__ bool gs_start(const GsDevIndex &I, const unsigned char *seq, int anchor,
                                         int dir, bool fwd, int KT, int iL, uint32_t &l,
                                         uint32_t &u, int &pos, bool &alive, bool &contained,
                                         unsigned long long &w_kmer, unsigned long long &w_blk)
{
    uint32_t pat = 0;
    int first_bad = KT;
#pragma unroll
    for (int j = 0; j < 16; j++) {
        if (j < KT) {
            unsigned char ch = seq[anchor + dir * j];
            uint32_t c = fwd ? gs_fwd_code(ch) : gs_comp_code(ch);
            if (c > 3u && first_bad == KT) first_bad = j;
            pat |= (c & 3u) << (j << 1);
        }
    }
    l = 1;
    u = 0;
    alive = false;
    contained = false;
    pos = anchor + dir * (GS_K0 - 1);
    if (first_bad < GS_K0) return false;
    w_kmer++;
    if (first_bad == KT) {
        if (KT == GS_K0) {
            uint2 iv = __ldg(&I.kmer[pat]);
            l = iv.x;
            u = iv.y;
            pos = anchor + dir * (KT - 1);
            alive = l <= u;
            return true;
        }
        uint2 iv = __ldg(&I.kmerx[pat]);
        uint32_t code = iv.y & 7u, size = iv.y >> 3;
        if (code != 7u) {
            l = iv.x;
            u = size ? iv.x + size - 1u : iv.x - 1u;
            pos = anchor + dir * (KT - 1);
            alive = size != 0;
            /* neighbour toward the longer match: e+1 (forward), s-1 (reverse) */
            int nb = anchor - dir;
            if (FORCED && alive && code < 4u && nb >= 0 && nb < iL) {
                unsigned char ch = seq[nb];
                uint32_t c = fwd ? gs_fwd_code(ch) : gs_comp_code(ch);
                contained = (c == code);
            }
            return true;
        }
        /* interval too wide to pack: the 13-mer start below */
    }
    uint2 iv = __ldg(&I.kmer[pat & ((1u << (2 * GS_K0)) - 1u)]);
    l = iv.x;
    u = iv.y;
    alive = l <= u;
    for (int j = GS_K0; j < KT && alive; j++) {
        int np = pos + dir;
        unsigned char ch = seq[np];
        uint32_t c = fwd ? gs_fwd_code(ch) : gs_comp_code(ch);
        if (c > 3u) {
            if (NSTOP) alive = false;
            else pos = np;
        } else {
            uint32_t nl = l, nu = u;
            w_blk += (unsigned long long)gs_step(I, nl, nu, c);
            if (nl > nu) {
                alive = false;
            } else {
                l = nl;
                u = nu;
                pos = np;
            }
        }
    }
    return true;
}

/* start-table length used for minimum seed length k */
__device__ __forceinline__ int gs_start_len(const GsDevIndex &I, int k)
{
    return (I.kx > GS_K0 && k > I.kx) ? I.kx : GS_K0;
}

/* ------------------------------------------------------------------ */
/* per-batch preparation: candidate slots and work items per read */

__global__ void gs_prepare_kernel(const uint32_t *lengths, uint32_t n_reads, int k,
                                  uint64_t *slot_n, uint32_t *item_n)
{
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r > n_reads) return;
    uint32_t n = 0;
    if (r < n_reads && lengths[r] >= (uint32_t)k) n = lengths[r] - (uint32_t)k + 1u;
    slot_n[r] = 2ull * n;
    item_n[r] = 2u * ((n + GS_CHUNK - 1) / GS_CHUNK);
}

int gs_launch_prepare(GsBatch &b, cudaStream_t st)
{
    uint32_t n = b.n_reads + 1;
    /* counts are written in place and scanned into offsets */
    gs_prepare_kernel<<<(n + 255) / 256, 256, 0, st>>>(b.lengths, b.n_reads, b.k, b.slot_off,
                                                        b.item_off);
    GS_CUDA(cudaGetLastError());
    return GS_OK;
}

/* ------------------------------------------------------------------ */
/* batched search */

/* one extension step of a candidate; false when it cannot extend further
 * (read end, empty interval, or a non-ACGT base under GS_N_STOP) */
template <int NSTOP>
__device__ __forceinline__ bool gs_advance(const GsDevIndex &I, const unsigned char *seq, int iL,
                                           bool fwd, int dir, uint32_t &l, uint32_t &u, int &pos)
{
    int np = pos + dir;
    if (np < 0 || np >= iL) return false;
    uint32_t c = fwd ? gs_fwd_code(seq[np]) : gs_comp_code(seq[np]);
    if (c > 3u) {
        if (NSTOP) return false;
        pos = np;   /* wildcard: interval unchanged */
        return true;
    }
    uint32_t nl = l, nu = u;
    gs_step(I, nl, nu, c);
    if (nl > nu) return false;
    l = nl;
    u = nu;
    pos = np;
    return true;
}

/* record of a finished candidate (seed_gen.cu:2259-2264, :2398-2404) */
__device__ __forceinline__ void gs_write_record(const GsBatch &B, uint32_t r, uint32_t n, bool fwd,
                                                int anchor, int pos, uint32_t l, uint32_t u,
                                                bool ok, bool killed)
{
    const int k = B.k;
    GsRec rec;
    rec.x = 0; rec.y = 0; rec.l = l; rec.u = u;
    if (!killed) {
        if (fwd) {
            /* length e - beg with beg = pos-1; a 13-mer that is absent still
             * counts 13 (the k == 13 case of :2259) */
            if (ok && anchor - pos + 1 >= k) {
                rec.x = pos;
                rec.y = anchor + 1;
            }
        } else if (ok && l <= u && pos + 1 - anchor >= k) {
            rec.x = (int32_t)((uint32_t)anchor | 0x80000000u);
            rec.y = (int32_t)((uint32_t)(pos + 1) | 0x80000000u);
        }
    }
    uint64_t slot = B.slot_off[r] + (fwd ? (uint64_t)(anchor - (k - 1)) : (uint64_t)n + (uint64_t)anchor);
    if (slot < B.slot_cap) B.slots[slot] = rec;
    else atomicOr(B.queue + 1, GS_FLAG_OVERFLOW);
}

template <int NSTOP>
__device__ __forceinline__ void gs_warp_item(const GsDevIndex &I, const GsBatch &B, uint32_t r,
                                             uint32_t local, int lane)
{
    const uint32_t L = B.lengths[r];
    const int k = B.k;
    const uint32_t n = L - (uint32_t)k + 1u;
    const uint32_t nch = (n + GS_CHUNK - 1) / GS_CHUNK;
    const bool fwd = local < nch;
    const uint32_t chunk = fwd ? local : local - nch;
    const uint32_t ci = chunk * GS_CHUNK + (uint32_t)lane;
    const bool in_range = ci < n;
    const bool owned = in_range && (lane < GS_CHUNK || ci == n - 1u);
    const unsigned char *seq = (const unsigned char *)B.seqs + B.offsets[r];
    const int iL = (int)L;

    /* anchor: e = k-1+ci (fwd), s = n-1-ci (rev); the containing neighbour
     * of every lane is lane+1 */
    int anchor = fwd ? (k - 1 + (int)ci) : ((int)n - 1 - (int)ci);
    const int dir = fwd ? -1 : 1;
    uint32_t l = 1, u = 0;
    int pos = anchor;
    bool alive = false, ok = false;
    unsigned long long wk = 0, wb = 0;
    bool killed = false;
    /* The start table's forced extensions are not used here.  A lockstep warp
     * lasts as long as its longest owned walk; a forced lane dies at step 1
     * by the neighbour rule anyway, and its step-1 size is what lane-1 is
     * compared with at step 1 (and lane 31, which nothing kills, is lane 30's
     * partner for the whole walk).  Stopping forced lanes at their start
     * saved 4% of the DRAM reads but, after keeping exactly those two
     * roles, still cost 2.5% of the time (config 3, 10M reads). */
    if (in_range) {
        bool contained = false;
        ok = gs_start<NSTOP, false>(I, seq, anchor, dir, fwd, gs_start_len(I, k), iL, l, u, pos,
                                    alive, contained, wk, wb);
    }

    uint32_t hist[GS_HIST];
#pragma unroll
    for (int m = 0; m < GS_HIST; m++) hist[m] = 0;
    uint32_t cur = alive ? u - l + 1u : 0u;
    int t = 0;
    const uint32_t owned_mask = __ballot_sync(0xffffffffu, owned);

    bool pushed = false;
    while (__ballot_sync(0xffffffffu, alive) & owned_mask) {
        if (alive) alive = gs_advance<NSTOP>(I, seq, iL, fwd, dir, l, u, pos);
        t++;
        uint32_t pub = alive ? u - l + 1u : 0u;
        /* containment: own size d steps ago vs the nearest extending lane
         * d to the right, which now stands at the same far end */
        uint32_t right = __ballot_sync(0xffffffffu, pub != 0u) & ~((2u << lane) - 1u);
        int j = right ? __ffs(right) - 1 : lane;
        uint32_t v = __shfl_sync(0xffffffffu, pub, j);
        int d = j - lane;
        if (alive && right && d <= GS_HIST && d <= t) {
            /* cur = own size one step ago, hist[m] = m+2 steps ago */
            uint32_t h = cur;
#pragma unroll
            for (int m = 0; m < GS_HIST - 1; m++) h = (d == m + 2) ? hist[m] : h;
            if (h == v) {
                alive = false;
                killed = true;
            }
        }
#pragma unroll
        for (int m = GS_HIST - 1; m > 0; m--) hist[m] = hist[m - 1];
        hist[0] = cur;
        cur = pub;
        /* few candidates left: hand them to the tail pass, which walks them
         * without lockstep, and free the warp */
        if (B.cont && t >= B.handoff_steps) {
            uint32_t left = __ballot_sync(0xffffffffu, alive) & owned_mask;
            if (__popc(left) <= B.handoff_lanes) {
                bool push = alive && owned;
                uint32_t base = 0;
                if (lane == 0 && left) base = atomicAdd(B.queue + 2, (uint32_t)__popc(left));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (push && base + __popc(left & ((1u << lane) - 1u)) >= B.cont_cap) {
                    atomicOr(B.queue + 1, GS_FLAG_OVERFLOW);
                    push = false;
                }
                if (push) {
                    GsCont cst;
                    cst.r = r;
                    cst.anchor = anchor;
                    cst.pos = pos;
                    cst.l = l;
                    cst.u = u;
                    cst.fwd = fwd ? 1u : 0u;
                    B.cont[base + __popc(left & ((1u << lane) - 1u))] = cst;
                    pushed = true;
                }
                break;
            }
        }
    }

    if (owned && !pushed) gs_write_record(B, r, n, fwd, anchor, pos, l, u, ok, killed);
}

/* Tail pass: the candidates handed over by gs_search_batched, one per lane;
 * a lane takes the next one as soon as its own is finished. */
template <int NSTOP>
__global__ void __launch_bounds__(256) gs_search_tail(GsDevIndex I, GsBatch B)
{
    const int lane = threadIdx.x & 31;
    uint32_t n_cont = *(volatile uint32_t *)(B.queue + 2);
    if (n_cont > B.cont_cap) n_cont = (uint32_t)B.cont_cap;
    bool have = false, exhausted = false;
    uint32_t r = 0, l = 0, u = 0, n = 0;
    int anchor = 0, pos = 0, iL = 0, dir = 0;
    bool fwd = false;
    const unsigned char *seq = NULL;
    for (;;) {
        uint32_t need = __ballot_sync(0xffffffffu, !have && !exhausted);
        if (need) {
            int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(B.queue + 3, (uint32_t)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!have && !exhausted) {
                uint32_t idx = base + __popc(need & ((1u << lane) - 1u));
                if (idx < n_cont) {
                    GsCont c = B.cont[idx];
                    r = c.r;
                    anchor = c.anchor;
                    pos = c.pos;
                    l = c.l;
                    u = c.u;
                    fwd = c.fwd != 0;
                    dir = fwd ? -1 : 1;
                    uint32_t L = B.lengths[r];
                    iL = (int)L;
                    n = L - (uint32_t)B.k + 1u;
                    seq = (const unsigned char *)B.seqs + B.offsets[r];
                    have = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__ballot_sync(0xffffffffu, have)) break;
        if (have && !gs_advance<NSTOP>(I, seq, iL, fwd, dir, l, u, pos)) {
            gs_write_record(B, r, n, fwd, anchor, pos, l, u, true, false);
            have = false;
        }
    }
}

template <int NSTOP>
__global__ void __launch_bounds__(256, 5) gs_search_batched(GsDevIndex I, GsBatch B, int queue_chunk)
{
    const int lane = threadIdx.x & 31;
    const uint32_t n_items = B.item_off[B.n_reads];
    if (n_items > B.item_cap) {
        /* the hand-over buffer was sized for fewer items (a captured pass
         * replayed on larger input): report, do nothing */
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(B.queue + 1, GS_FLAG_OVERFLOW);
        return;
    }
    for (;;) {
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(B.queue, (uint32_t)queue_chunk);
        first = __shfl_sync(0xffffffffu, first, 0);
        if (first >= n_items) break;
        uint32_t last = min(first + (uint32_t)queue_chunk, n_items);
        /* read of the first item: largest r with item_off[r] <= first */
        uint32_t lo = 0, hi = B.n_reads;
        while (lo + 1 < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (B.item_off[mid] <= first) lo = mid; else hi = mid;
        }
        uint32_t r = lo;
        for (uint32_t it = first; it < last; it++) {
            while (B.item_off[r + 1] <= it) r++;
            gs_warp_item<NSTOP>(I, B, r, it - B.item_off[r], lane);
        }
    }
}

/* ------------------------------------------------------------------ */
/* plain search: one read per thread */

template <int NSTOP>
__global__ void __launch_bounds__(128) gs_search_plain(GsDevIndex I, GsBatch B)
{
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B.n_reads) return;
    const uint32_t L = B.lengths[r];
    const int k = B.k;
    if (L < (uint32_t)k) return;
    const uint32_t n = L - (uint32_t)k + 1u;
    const unsigned char *seq = (const unsigned char *)B.seqs + B.offsets[r];
    uint32_t *H = B.hist + B.offsets[r];
    GsRec *slots = B.slots + B.slot_off[r];
    const int iL = (int)L;
    unsigned long long w_kmer = 0, w_blk = 0;
    const int KT = gs_start_len(I, k);

    for (int strand = 0; strand < 2; strand++) {
        const bool fwd = strand == 0;
        for (uint32_t q = 0; q < L; q++) H[q] = 0;
        for (uint32_t ci = 0; ci < n; ci++) {
            /* forward: e from L-1 down; reverse: s from 0 up */
            int anchor = fwd ? iL - 1 - (int)ci : (int)ci;
            const int dir = fwd ? -1 : 1;
            uint32_t l = 1, u = 0;
            int pos = anchor;
            bool alive = false;
            bool contained = false;
            bool ok = gs_start<NSTOP, true>(I, seq, anchor, dir, fwd, KT, iL, l, u, pos, alive, contained,
                                      w_kmer, w_blk);
            bool killed = contained;
            if (contained) {
                /* it reached its start level: the candidates to its left may
                 * compare with it there */
                H[pos] = u - l + 1u;
                alive = false;
            }
            if (alive) {
                uint32_t sz = u - l + 1u;
                uint32_t h = H[pos];
                H[pos] = sz;
                killed = (h == sz);
                while (!killed) {
                    int np = pos + dir;
                    if (np < 0 || np >= iL) break;
                    uint32_t c = fwd ? gs_fwd_code(seq[np]) : gs_comp_code(seq[np]);
                    uint32_t nl = l, nu = u;
                    if (c > 3u) {
                        if (NSTOP) break;
                    } else {
                        w_blk += (unsigned long long)gs_step(I, nl, nu, c);
                        if (nl > nu) break;
                    }
                    l = nl;
                    u = nu;
                    pos = np;
                    sz = u - l + 1u;
                    h = H[pos];
                    H[pos] = sz;
                    killed = (h == sz);
                }
            }
            GsRec rec;
            rec.x = 0; rec.y = 0; rec.l = l; rec.u = u;
            if (!killed && ok) {
                if (fwd) {
                    if (anchor - pos + 1 >= k) { rec.x = pos; rec.y = anchor + 1; }
                } else if (l <= u && pos + 1 - anchor >= k) {
                    rec.x = (int32_t)((uint32_t)anchor | 0x80000000u);
                    rec.y = (int32_t)((uint32_t)(pos + 1) | 0x80000000u);
                }
            }
            uint64_t slot = fwd ? (uint64_t)(anchor - (k - 1)) : (uint64_t)n + (uint64_t)anchor;
            slots[slot] = rec;
        }
    }
    if (B.work) {
        atomicAdd(&B.work[0], w_kmer);
        atomicAdd(&B.work[1], w_blk);
    }
}

/* ------------------------------------------------------------------ */

int gs_launch_search(const GsDevIndex &I, GsBatch &B, int kernel, int queue_chunk, int ctas_per_sm,
                     uint32_t n_items, cudaStream_t st)
{
    if (B.n_reads == 0) return GS_OK;
    if (kernel == GS_KERNEL_PLAIN) {
        uint32_t nb = (B.n_reads + 127) / 128;
        if (B.n_mode == GS_N_STOP) gs_search_plain<1><<<nb, 128, 0, st>>>(I, B);
        else gs_search_plain<0><<<nb, 128, 0, st>>>(I, B);
        GS_CUDA(cudaGetLastError());
        return GS_OK;
    }
    int dev = 0, sms = 0;
    GS_CUDA(cudaGetDevice(&dev));
    GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (queue_chunk <= 0) queue_chunk = GS_QUEUE_CHUNK;
    if (ctas_per_sm <= 0) {
        int occ = 0;
        if (B.n_mode == GS_N_STOP)
            GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gs_search_batched<1>, 256, 0));
        else
            GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gs_search_batched<0>, 256, 0));
        ctas_per_sm = occ > 0 ? occ : 1;
    }
    uint32_t grid = (uint32_t)sms * (uint32_t)ctas_per_sm;
    if (n_items) {
        uint32_t need = (n_items + (uint32_t)queue_chunk - 1) / (uint32_t)queue_chunk;
        uint32_t warps = grid * 8;
        if (need < warps) grid = (need + 7) / 8;
    }
    if (grid == 0) grid = 1;
    GS_CUDA(cudaMemsetAsync(B.queue, 0, sizeof(uint32_t), st));
    if (B.cont) GS_CUDA(cudaMemsetAsync(B.queue + 2, 0, 2 * sizeof(uint32_t), st));
    if (B.n_mode == GS_N_STOP) gs_search_batched<1><<<grid, 256, 0, st>>>(I, B, queue_chunk);
    else gs_search_batched<0><<<grid, 256, 0, st>>>(I, B, queue_chunk);
    GS_CUDA(cudaGetLastError());
    if (B.cont) {
        int tocc = 0;
        if (B.n_mode == GS_N_STOP)
            GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tocc, gs_search_tail<1>, 256, 0));
        else
            GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tocc, gs_search_tail<0>, 256, 0));
        uint32_t tgrid = (uint32_t)sms * (uint32_t)(tocc > 0 ? tocc : 4);
        if (B.n_mode == GS_N_STOP) gs_search_tail<1><<<tgrid, 256, 0, st>>>(I, B);
        else gs_search_tail<0><<<tgrid, 256, 0, st>>>(I, B);
        GS_CUDA(cudaGetLastError());
    }
    return GS_OK;
}
