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
 * flags (:2100-2204); this file uses a defined rule with three launch forms:
 *
 *   GS_KERNEL_BATCHED (default): gs_search_start + gs_search_walk (+
 *     gs_search_text, gs_search_leftover).  Each candidate carries the
 *     interval of its neighbour's string at its own far end and stops
 *     exactly where the rule says; candidates are started a warp per work
 *     item and walked one per lane (see "batched search").
 *   GS_KERNEL_LOCKSTEP: gs_search_lockstep + gs_search_tail.  Persistent
 *     CTAs; each warp takes work items (read, strand, 31 candidates + 1
 *     helper lane) from a global queue and steps its 32 candidates in
 *     lockstep, comparing with the nearest still-extending lane to the right
 *     from a GS_HIST-deep own history; the last candidates of a warp go to a
 *     tail pass.
 *   GS_KERNEL_PLAIN: gs_search_plain, one thread per read, candidates one
 *     after another, containment history in a per-read global array.
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

/* Longer start table, built in four passes over all kx-mers (base j at
 * bits 2j, processed first, i.e. the string's last character sits at bits
 * 0-1):
 *   1. (l,u) from the 13-mer prefix interval plus kx-13 steps;
 *   2. the forced right extension of each kx-mer X: the base c with
 *      count(Xc) == count(X) > 0, if any.  Xc's interval is one step with X's
 *      first character from the kx-mer table entry of (X without its first
 *      character)·c;
 *   3. packing: entry.x = l, entry.y = size << 3 | code, code 0-3 the forced
 *      base, 4 none, 7 "size does not fit 29 bits: start from the 13-mer";
 *   4. entry.z, entry.w = the packed entry of gs_kmer_rc(X), the kx-mer of
 *      X's reverse complement in the same bit order.
 * A candidate whose kx-mer is always followed by its neighbour's next base is
 * contained in that neighbour (see the file comment) and needs no walk;
 * gs_search_plain stops such candidates at their start.  A read's window
 * R[s..s+kx-1] is the start string of its forward candidate ending at
 * s+kx-1 and, as complement codes, of its reverse candidate starting at s:
 * the two keys are X and gs_kmer_rc(X), so one 16-byte entry starts both. */
__device__ __forceinline__ uint32_t gs_kmer_rc(uint32_t X, int kx)
{
    /* complement every base (3 - c = c ^ 3), then reverse the order of the
     * kx 2-bit groups */
    const uint32_t b = __brev(~X);
    return (((b >> 1) & 0x55555555u) | ((b & 0x55555555u) << 1)) >> (32 - 2 * kx);
}

__global__ void gs_kmerx_kernel(GsDevIndex I, uint4 *table, int kx, uint64_t n)
{
    for (uint64_t patt = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; patt < n;
         patt += (uint64_t)gridDim.x * blockDim.x) {
        uint2 iv = __ldg(&I.kmer[patt & ((1u << (2 * GS_K0)) - 1u)]);
        uint32_t l = iv.x, u = iv.y;
        for (int i = GS_K0; i < kx && l <= u; i++) gs_step(I, l, u, (uint32_t)(patt >> (i << 1)) & 3u);
        table[patt] = make_uint4(l, u, 0u, 0u);
    }
}

__global__ void gs_kmerx_code_kernel(GsDevIndex I, const uint4 *table, int kx, uint64_t n,
                                     uint8_t *code)
{
    const uint64_t mask = n - 1;
    for (uint64_t X = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; X < n;
         X += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 e4 = table[X];
        const uint2 e = make_uint2(e4.x, e4.y);
        uint8_t out = 4;
        if (e.x <= e.y) {
            uint32_t size = e.y - e.x + 1u;
            uint32_t first = (uint32_t)(X >> (2 * (kx - 1))) & 3u;   /* X's first character */
            for (uint32_t c = 0; c < 4; c++) {
                const uint4 y4 = table[((X << 2) | c) & mask];
                const uint2 y = make_uint2(y4.x, y4.y);
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

__global__ void gs_kmerx_pack_kernel(uint4 *table, uint64_t n, const uint8_t *code)
{
    for (uint64_t X = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; X < n;
         X += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 e = table[X];
        uint32_t size = e.x <= e.y ? e.y - e.x + 1u : 0u;
        uint32_t c = code[X];
        if (size >= (1u << 29)) {
            size = 0;
            c = 7;
        }
        table[X] = make_uint4(e.x, (size << 3) | c, 0u, 0u);
    }
}

/* pass 4: each entry's second half from the packed first half of its
 * reverse complement's entry (reads only x,y and writes only z,w) */
__global__ void gs_kmerx_pair_kernel(uint4 *table, int kx, uint64_t n)
{
    uint2 *w = reinterpret_cast<uint2 *>(table);
    for (uint64_t X = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; X < n;
         X += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 rc = w[2 * (uint64_t)gs_kmer_rc((uint32_t)X, kx)];
        w[2 * X + 1] = rc;
    }
}

int gs_build_kmerx_table(const GsDevIndex &I, uint4 *table, int kx, cudaStream_t st)
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
    if (e == cudaSuccess) {
        gs_kmerx_pair_kernel<<<152 * 64, 256, 0, st>>>(table, kx, n);
        e = cudaGetLastError();
    }
    cudaFreeAsync(code, st);
    if (e != cudaSuccess) return gs_cuda_fail(e, "k-mer start table");
    return GS_OK;
}

/* a start-table entry: one random 8-byte load whose L2 fill is 64 bytes
 * (the default fills 128 for random loads; the table's lookups are bound by
 * the DRAM access rate, and the start pass also streams the walker buffer) */
__device__ __forceinline__ uint2 gs_ld_entry(const uint2 *p)
{
    uint2 v;
    asm("ld.global.nc.L2::64B.v2.u32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

/* both halves of a paired start-table entry: one 16-byte load, the same
 * 64-byte L2 fill */
__device__ __forceinline__ uint4 gs_ld_pair(const uint4 *p)
{
    uint4 v;
    asm("ld.global.nc.L2::64B.v4.u32 {%0,%1,%2,%3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p));
    return v;
}

/* The start from the 13-mer table: the interval of the first 13 bases,
 * then steps up to KT bases (a non-ACGT base is a wildcard, or stops the
 * start under GS_N_STOP) */
template <int NSTOP>
__device__ __forceinline__ void gs_start_from13(const GsDevIndex &I, const unsigned char *seq,
                                                int anchor, int dir, bool fwd, int KT, uint32_t pat,
                                                uint32_t &l, uint32_t &u, int &pos, bool &alive,
                                                unsigned long long &w_blk)
{
    uint2 iv = gs_ld_entry(&I.kmer[pat & ((1u << (2 * GS_K0)) - 1u)]);
    l = iv.x;
    u = iv.y;
    alive = l <= u;
    pos = anchor + dir * (GS_K0 - 1);
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
}

/* Start of a candidate: the interval of its first KT bases (forward: the
 * bases anchor, anchor-1, ...; reverse: the complement codes anchor,
 * anchor+1, ...; the first base at bits 0-1).  Returns false when one of the
 * first 13 bases is not ACGT (no search, seed_gen.cu:2132-2143).  A non-ACGT
 * base at positions 13..KT-1 takes the 13-mer start and steps over it like
 * the main loop does.  pos = far end reached; alive = interval non-empty;
 * contained (FORCED only) = the start string is always followed by the
 * neighbour's next base (the candidate needs no walk and produces no record);
 * fcode = the start table's forced-extension code (0-3, or 4: none/unknown). */
template <int NSTOP, bool FORCED>
__device__ __forceinline__ bool gs_start(const GsDevIndex &I, const unsigned char *seq, int anchor,
                                         int dir, bool fwd, int KT, int iL, uint32_t &l,
                                         uint32_t &u, int &pos, bool &alive, bool &contained,
                                         uint32_t &fcode, unsigned long long &w_kmer,
                                         unsigned long long &w_blk)
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
    fcode = 4;
    pos = anchor + dir * (GS_K0 - 1);
    if (first_bad < GS_K0) return false;
    w_kmer++;
    if (first_bad == KT) {
        if (KT == GS_K0) {
            uint2 iv = gs_ld_entry(&I.kmer[pat]);
            l = iv.x;
            u = iv.y;
            pos = anchor + dir * (KT - 1);
            alive = l <= u;
            return true;
        }
        uint2 iv = gs_ld_entry(reinterpret_cast<const uint2 *>(&I.kmerx[pat]));
        uint32_t code = iv.y & 7u, size = iv.y >> 3;
        if (code != 7u) {
            fcode = code;
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
    gs_start_from13<NSTOP>(I, seq, anchor, dir, fwd, KT, pat, l, u, pos, alive, w_blk);
    return true;
}

/* start-table length used for minimum seed length k */
__host__ __device__ __forceinline__ int gs_start_len(const GsDevIndex &I, int k)
{
    return (I.kx > GS_K0 && k > I.kx) ? I.kx : GS_K0;
}

/* one candidate's start as gs_start reports it */
struct GsStart {
    uint32_t l, u, fcode;
    int pos;
    bool ok, alive;
};

/* a start from one packed half of a start-table entry; false for code 7
 * (interval too wide to pack: the caller starts from the 13-mer) */
__device__ __forceinline__ bool gs_entry_start(uint32_t x, uint32_t y, int anchor, int dir, int KT,
                                               GsStart &S)
{
    const uint32_t code = y & 7u, size = y >> 3;
    if (code == 7u) return false;
    S.fcode = code;
    S.l = x;
    S.u = size ? x + size - 1u : x - 1u;
    S.pos = anchor + dir * (KT - 1);
    S.alive = size != 0;
    return true;
}

/* gs_start of one candidate: the rare starts of a paired window (a
 * non-ACGT base in it, or an interval too wide to pack) */
template <int NSTOP>
__device__ __forceinline__ GsStart gs_start_apart(const GsDevIndex &I, const unsigned char *seq,
                                               int anchor, bool fwd, int KT, int iL)
{
    GsStart S;
    bool contained;
    unsigned long long w_kmer = 0, w_blk = 0;
    S.ok = gs_start<NSTOP, false>(I, seq, anchor, fwd ? -1 : 1, fwd, KT, iL, S.l, S.u, S.pos,
                                  S.alive, contained, S.fcode, w_kmer, w_blk);
    return S;
}

/* Both candidates of read window R[s..s+KT-1] (KT = I.kx): the forward one
 * ending at s+KT-1 (vf) and the reverse one starting at s (vr), with the
 * same results as gs_start on each.  An ACGT-only window takes one paired
 * entry for both; a window with another base starts each candidate on its
 * own (the 13-mer rule and the wildcard steps depend on where the base
 * lies in each walk order). */
template <int NSTOP>
__device__ __forceinline__ void gs_start_pair(const GsDevIndex &I, const unsigned char *seq, int s,
                                              int KT, int iL, bool vf, bool vr, GsStart &F,
                                              GsStart &R, unsigned long long &w_kmer,
                                              unsigned long long &w_blk)
{
    const int ef = s + KT - 1;
    F.l = R.l = 1u;
    F.u = R.u = 0u;
    F.fcode = R.fcode = 4u;
    F.ok = R.ok = F.alive = R.alive = false;
    F.pos = ef - (GS_K0 - 1);
    R.pos = s + (GS_K0 - 1);
    if (!vf && !vr) return;
    /* the reverse key: complement codes, R[s] at bits 0-1 */
    uint32_t pr = 0;
    bool bad = false;
#pragma unroll
    for (int j = 0; j < 16; j++) {
        if (j < KT) {
            const uint32_t c = gs_comp_code(seq[s + j]);
            bad |= c > 3u;
            pr |= (c & 3u) << (j << 1);
        }
    }
    if (!bad) {
        /* the forward key (R[s+KT-1] at bits 0-1) is pr's reverse complement */
        const uint32_t pf = gs_kmer_rc(pr, KT);
        const uint4 e = gs_ld_pair(&I.kmerx[pf]);
        /* code 7 (interval too wide to pack): gs_start's own 13-mer start */
        bool wide = false;
        if (vf) {
            F.ok = true;
            wide = !gs_entry_start(e.x, e.y, ef, -1, KT, F);
        }
        if (vr) {
            R.ok = true;
            wide |= !gs_entry_start(e.z, e.w, s, 1, KT, R);
        }
        if (!wide) {
            w_kmer++;
            return;
        }
    }
    /* (the work counters count one lookup per candidate here) */
    if (vf) {
        F = gs_start_apart<NSTOP>(I, seq, ef, true, KT, iL);
        w_kmer++;
    }
    if (vr) {
        R = gs_start_apart<NSTOP>(I, seq, s, false, KT, iL);
        w_kmer++;
    }
}

/* ------------------------------------------------------------------ */
/* per-batch preparation: candidate slots and work items per read */

__global__ void gs_prepare_kernel(const uint32_t *lengths, uint32_t n_reads, int k, int paired_kt,
                                  uint64_t *slot_n, uint32_t *item_n)
{
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r > n_reads) return;
    uint32_t n = 0;
    if (r < n_reads && lengths[r] >= (uint32_t)k) n = lengths[r] - (uint32_t)k + 1u;
    slot_n[r] = 2ull * n;
    if (paired_kt) {
        /* windows s in [0, L-KT] (k >= KT, so L-KT+1 >= n) */
        const uint32_t w = n ? lengths[r] - (uint32_t)paired_kt + 1u : 0u;
        item_n[r] = (w + GS_PCHUNK - 1) / GS_PCHUNK;
    } else {
        item_n[r] = 2u * ((n + GS_CHUNK - 1) / GS_CHUNK);
    }
}

int gs_launch_prepare(const GsDevIndex &I, GsBatch &b, int kernel, cudaStream_t st)
{
    uint32_t n = b.n_reads + 1;
    /* the batched start pass pairs each window's two candidates when it
     * starts from the longer table */
    b.paired = kernel == GS_KERNEL_BATCHED && I.kx > GS_K0 && gs_start_len(I, b.k) == I.kx;
    /* counts are written in place and scanned into offsets */
    gs_prepare_kernel<<<(n + 255) / 256, 256, 0, st>>>(b.lengths, b.n_reads, b.k,
                                                        b.paired ? I.kx : 0, b.slot_off,
                                                        b.item_off);
    GS_CUDA(cudaGetLastError());
    return GS_OK;
}

/* ------------------------------------------------------------------ */
/* lockstep search */

/* one extension step of a candidate; false when it cannot extend further
 * (read end, empty interval, or a non-ACGT base under GS_N_STOP) */
template <int NSTOP, int COUNT>
__device__ __forceinline__ bool gs_advance(const GsDevIndex &I, const unsigned char *seq, int iL,
                                           bool fwd, int dir, uint32_t &l, uint32_t &u, int &pos,
                                           unsigned long long &w_blk)
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
    int blocks = gs_step(I, nl, nu, c);
    if (COUNT) w_blk += (unsigned long long)blocks;
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
    if (rec.y == 0) return;   /* no record: the slot stays unflagged and unwritten */
    uint64_t slot = B.slot_off[r] + (fwd ? (uint64_t)(anchor - (k - 1)) : (uint64_t)n + (uint64_t)anchor);
    if (slot < B.slot_cap) {
        B.slots[slot] = rec;
        atomicOr(B.recmask + (slot >> 5), 1u << (slot & 31u));
    } else {
        atomicOr(B.queue + 1, GS_FLAG_OVERFLOW);
    }
}

template <int NSTOP, int COUNT>
__device__ __forceinline__ void gs_lockstep_item(const GsDevIndex &I, const GsBatch &B, uint32_t r,
                                             uint32_t local, int lane, unsigned long long &wk,
                                             unsigned long long &wb)
{
    const uint32_t L = B.lengths[r];
    const int k = B.k;
    const uint32_t n = L - (uint32_t)k + 1u;
    const uint32_t nch = (n + GS_CHUNK - 1) / GS_CHUNK;
    const bool fwd = local < nch;
    const uint32_t chunk = fwd ? local : local - nch;
    const uint32_t ci = chunk * GS_CHUNK + (uint32_t)lane;
    const bool in_range = ci < n;
    /* lane 31 only starts the next item's first candidate (which that item
     * owns: ceil(n / GS_CHUNK) items cover every candidate) */
    const bool owned = in_range && lane < GS_CHUNK;
    const unsigned char *seq = (const unsigned char *)B.seqs + B.offsets[r];
    const int iL = (int)L;

    /* anchor: e = k-1+ci (fwd), s = n-1-ci (rev); the containing neighbour
     * of every lane is lane+1 */
    int anchor = fwd ? (k - 1 + (int)ci) : ((int)n - 1 - (int)ci);
    const int dir = fwd ? -1 : 1;
    uint32_t l = 1, u = 0;
    int pos = anchor;
    bool alive = false, ok = false;
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
        uint32_t fcode = 4;
        ok = gs_start<NSTOP, false>(I, seq, anchor, dir, fwd, gs_start_len(I, k), iL, l, u, pos,
                                    alive, contained, fcode, wk, wb);
    }

    uint32_t hist[GS_HIST];
#pragma unroll
    for (int m = 0; m < GS_HIST; m++) hist[m] = 0;
    uint32_t cur = alive ? u - l + 1u : 0u;
    int t = 0;
    const uint32_t owned_mask = __ballot_sync(0xffffffffu, owned);

    bool pushed = false;
    while (__ballot_sync(0xffffffffu, alive) & owned_mask) {
        if (alive) alive = gs_advance<NSTOP, COUNT>(I, seq, iL, fwd, dir, l, u, pos, wb);
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

/* executed-work counters (count_work with the batched kernel): a warp sum,
 * one atomic per warp */
__device__ __forceinline__ void gs_add_work(const GsBatch &B, unsigned long long wk,
                                            unsigned long long wb)
{
    for (int o = 16; o > 0; o >>= 1) {
        wk += __shfl_xor_sync(0xffffffffu, wk, o);
        wb += __shfl_xor_sync(0xffffffffu, wb, o);
    }
    if ((threadIdx.x & 31) == 0 && B.work) {
        atomicAdd(&B.work[0], wk);
        atomicAdd(&B.work[1], wb);
    }
}

/* Tail pass: the candidates handed over by gs_search_lockstep, one per lane;
 * a lane takes the next one as soon as its own is finished. */
template <int NSTOP, int COUNT>
__global__ void __launch_bounds__(256) gs_search_tail(GsDevIndex I, GsBatch B)
{
    const int lane = threadIdx.x & 31;
    unsigned long long wb = 0;
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
        if (have && !gs_advance<NSTOP, COUNT>(I, seq, iL, fwd, dir, l, u, pos, wb)) {
            gs_write_record(B, r, n, fwd, anchor, pos, l, u, true, false);
            have = false;
        }
    }
    if (COUNT) gs_add_work(B, 0, wb);
}

template <int NSTOP, int COUNT>
__global__ void __launch_bounds__(256, 5) gs_search_lockstep(GsDevIndex I, GsBatch B, int queue_chunk)
{
    const int lane = threadIdx.x & 31;
    unsigned long long wk = 0, wb = 0;
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
            gs_lockstep_item<NSTOP, COUNT>(I, B, r, it - B.item_off[r], lane, wk, wb);
        }
    }
    if (COUNT) gs_add_work(B, wk, wb);
}

/* ------------------------------------------------------------------ */
/* batched search
 *
 * Candidate e is contained in e+1 at far end p exactly when
 * count(R[p..e]) == count(R[p..e+1]) (sizes only fall along the chain
 * e, e+1, ..., so this is the nearest-extending-candidate rule of the file
 * comment).  R[p..e+1]'s interval J is nested in R[p..e]'s interval I, so a
 * candidate can carry J itself and stop at the canonical step without
 * seeing its neighbour: no lockstep, no helper lane walking, no history.
 * J's bounds share occurrence blocks with I's whenever I is narrow.
 *
 *   gs_search_start: a warp per work item, one round of start-table
 *     lookups.  With the longer start table (k > kx) an item is 30 read
 *     windows (+ a helper window on each side) and one paired entry starts
 *     a window's forward and reverse candidate (gs_start_pair_item); else
 *     31 candidates of one strand + the next item's first, started for its
 *     interval only (gs_start_item).  The forced-extension code settles J
 *     where it can (forced to the neighbour's base: contained, stop; forced
 *     elsewhere: no J); otherwise the walker carries its neighbour's start
 *     interval and its first step in the walk pass extends that to I's far
 *     end.  Survivors go to the walker buffer in per-warp reserved chunks
 *     (unused entries marked r = ~0); a walker that finds the buffer full is
 *     left in its record slot for gs_search_leftover.
 *   gs_search_walk: one walker per lane, each lane refilled as soon as its
 *     walker ends, from a per-warp window of the buffer; walkers that reach
 *     one row without J go to gs_search_text. */

#define GS_WALKER_HOLE 0xffffffffu
#define GS_WALKER_JPEND 0x40000000u   /* anchor flag: J is one base short of I's far end */
#define GS_WALKER_FWD 0x80000000u
#define GS_WALKER_CHUNK 512u      /* most buffer entries a warp reserves at a time */

/* entries a start-pass warp reserves at a time (gs_launch_batched sets it) */
__device__ __forceinline__ uint32_t gs_walker_chunk(const GsBatch &B)
{
    return B.walker_chunk;
}

/* Sizes from the walker buffer's capacity and a grid of `warps` warps,
 * multiples of 32 from 32 to `most`: about 1/`parts` of a warp's share, so
 * that a small batch's buffer (start reservations) or walkers (walk-pass
 * windows) spread over every warp */
static uint32_t gs_share_size(uint64_t cap, uint32_t warps, uint32_t parts, uint32_t most)
{
    uint64_t v = cap / ((uint64_t)warps * parts);
    v &= ~31ull;
    if (v < 32u) v = 32u;
    if (v > most) v = most;
    return (uint32_t)v;
}
#define GS_WALK_WINDOW 512u       /* most buffer entries a walk-pass warp takes at a time */

/* Text mode.  A walker whose interval is one row [l,l] and whose J is
 * empty can no longer be contained: its walk only extends one occurrence,
 * at text position q = SA[l], while the read goes on matching T[q-1],
 * T[q-2], ...  It ends where the read and the text differ, the read or the
 * text ends, or (GS_N_STOP) a non-ACGT base comes; its record is the row of
 * the suffix at that position.  Text mode finds that position by comparing
 * 16 bases a round and takes its row from the inverse-SA sample at or above
 * it, with at most GS_ISA_STEP-1 LF steps over the text bases in between.
 * Under GS_N_WILDCARD a non-ACGT base hands the walker back to the
 * interval walk, which skips the base.  The walker's J words hold the
 * state: jl = GS_TEXT_MARK | phase << 26 | flags, ju = a text position. */
#define GS_TM_MOVED (1u << 25)   /* the compare advanced past the entry position */
#define GS_TM_CONT (1u << 24)    /* a wildcard base follows: back to the interval walk */

/* The 2-bit codes (forward or complement table) and the non-ACGT flags of 4
 * ASCII bytes: a byte-permute lookup of the nibble table, indexed by ch & 7 */
__device__ __forceinline__ void gs_codes4(uint32_t b, bool fwd, uint32_t &packed, uint32_t &inv)
{
    const uint32_t idx = b & 0x07070707u;
    const uint32_t sel = (idx & 7u) | ((idx >> 4) & 0x70u) | ((idx >> 8) & 0x700u) |
                         ((idx >> 12) & 0x7000u);
    /* bytes 0..7 = code of ch & 7: forward A0 C1 G2 T3 N4 others 0/5, complement */
    const uint32_t c = fwd ? __byte_perm(0x01000005u, 0x02040003u, sel)
                           : __byte_perm(0x02000305u, 0x01040000u, sel);
    uint32_t v = c & 0x03030303u;
    v = (v | (v >> 6)) & 0x000f000fu;
    packed = (v | (v >> 12)) & 0xffu;
    uint32_t iv = (c >> 2) & 0x01010101u;   /* codes 4 and 5 */
    iv = (iv | (iv >> 7)) & 0x00030003u;
    inv = (iv | (iv >> 14)) & 0xfu;
}

/* The read's next `avail` (1..16) bases in walk order from pos: the first at
 * bits 30-31 of *wr (2-bit codes), and *inv with bit 31 - i set when the
 * i-th is not ACGT.  Loads the aligned words that hold the bytes, each of
 * which holds at least one byte of the read. */
__device__ __forceinline__ void gs_read_window(const unsigned char *seq, int pos, bool fwd,
                                               int avail, uint32_t &wr, uint32_t &inv32)
{
    const unsigned char *lo = seq + (fwd ? pos - avail : pos + 1);
    const uintptr_t a = (uintptr_t)lo;
    const uint32_t *wp = (const uint32_t *)(a & ~(uintptr_t)3);
    const uint32_t off = (uint32_t)(a & 3u);
    const uint32_t nw = (off + (uint32_t)avail + 3u) >> 2;   /* 1..5 */
    uint32_t w[5];
#pragma unroll
    for (int k = 0; k < 5; k++) w[k] = (uint32_t)k < nw ? __ldg(wp + k) : 0u;
    uint32_t wr16 = 0, inv16 = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint32_t p, iv;
        gs_codes4(__funnelshift_r(w[k], w[k + 1], off * 8u), fwd, p, iv);
        wr16 |= p << (8 * k);
        inv16 |= iv << (4 * k);
    }
    if (fwd) {
        /* memory order ends with the first base of the walk (pos-1) */
        wr = wr16 << (2 * (16 - avail));
        inv32 = inv16 << (32 - avail);
    } else {
        /* memory order starts with it (pos+1): reverse the 2-bit groups */
        uint32_t x = __brev(wr16);
        wr = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
        inv32 = __brev(inv16) & (0xffffffffu << (32 - avail));
    }
}

template <int COUNT>
__device__ __forceinline__ bool gs_text_round(const GsDevIndex &I, const unsigned char *seq, int iL,
                                              bool fwd, int dir, uint32_t &l, uint32_t &u,
                                              uint32_t &jl, uint32_t &ju, int &pos, int nstop,
                                              unsigned long long &wb)
{
    const uint32_t ph = (jl >> 26) & 3u;
    (void)wb;
    if (ph == 0) {
        ju = gs_ld64(&I.saf[l]);
        jl = GS_TEXT_MARK | (1u << 26);
        return true;
    }
    bool cont;
    if (ph == 1) {
        const uint32_t q = ju;
        const int rem = fwd ? pos : iL - 1 - pos;
        int avail = rem < 16 ? rem : 16;
        if ((uint32_t)avail > q) avail = (int)q;
        int m = 0, bad = avail;
        if (avail > 0) {
            /* T[q-16..q-1], T[q-1] at bits 30-31 */
            uint32_t wt;
            if (q >= 16) {
                const uint32_t b = q - 16u;
                wt = __funnelshift_r(gs_ld64(&I.text[b >> 4]), gs_ld64(&I.text[(b >> 4) + 1]),
                                     (b & 15u) << 1);
            } else {
                wt = __ldg(&I.text[0]) << ((16u - q) << 1);
            }
            /* the read's next bases in walk order, the first at bits 30-31 */
            uint32_t wr, inv32;
            gs_read_window(seq, pos, fwd, avail, wr, inv32);
            if (inv32) bad = __clz(inv32);
            m = (int)(__clz(wr ^ wt) >> 1);
            if (m > bad) m = bad;
            pos += dir * m;
            ju = q - (uint32_t)m;
            if (m) jl |= GS_TM_MOVED;
            if (m == avail && avail < rem && ju > 0u) return true;
        }
        cont = !nstop && m == bad && bad < avail;
        if (!(jl & GS_TM_MOVED)) {
            /* still at the entry row */
            if (!cont) return false;
            jl = 1u;
            ju = 0u;
            return true;
        }
        jl = GS_TEXT_MARK | (2u << 26) | (cont ? GS_TM_CONT : 0u);
        return true;
    }
    cont = (jl & GS_TM_CONT) != 0;
    {
        /* the row of position qs from the sample at qp >= qs (position
         * seq_len is row 0), and T[qs..qs+3] for the LF steps down to qs */
        const uint32_t qs = ju;
        uint32_t qp = (qs + GS_ISA_STEP - 1u) & ~(GS_ISA_STEP - 1u);
        uint32_t row = 0;
        if (qp > I.seq_len) qp = I.seq_len;
        else row = gs_ld64(&I.isa[qp / GS_ISA_STEP]);
        const uint32_t w = __funnelshift_r(gs_ld64(&I.text[qs >> 4]), gs_ld64(&I.text[(qs >> 4) + 1]),
                                           (qs & 15u) << 1);
        l = u = row;
        const uint32_t d = qp - qs;
        jl = GS_TEXT_MARK | (3u << 26) | (jl & GS_TM_CONT) | (d << 16) | (w & 0xffu);
        if (d) return true;
    }
    /* phase 3, the LF steps, is the interval walk's own step (gs_walk_step) */
    if (!cont) return false;
    jl = 1u;
    ju = 0u;
    return true;
}

/* One iteration of a walk: normally a step of I and J with the next
 * base; for a walker whose J is still one base short (jpend), the J-only
 * step with the base at pos that brings J to I's far end -- the same call,
 * so the lanes of a warp take one memory round per iteration either way.
 * Returns false when the walk is over (killed: it ended by containment).
 * A step that leaves the walker eligible for text mode sets jl to
 * GS_TEXT_MARK. */
/* walk-pass counters of a count_work pass (gs_ctx_last_walk_counts) */
struct GsWalkCounts {
    unsigned long long steps, jsteps, jblocks, jshrank, jwalkers, lines256, lines384;
};

template <int NSTOP, int COUNT, bool TEXT>
__device__ __forceinline__ bool gs_walk_step(const GsDevIndex &I, const unsigned char *seq, int iL,
                                             bool fwd, int dir, uint32_t &l, uint32_t &u,
                                             uint32_t &jl, uint32_t &ju, int &pos, bool &jpend,
                                             bool &killed, unsigned long long &wb,
                                             GsWalkCounts *wc = nullptr)
{
    /* TEXT: text-mode states run here; otherwise the caller hands a walker
     * that enters text mode to the text pass */
    const bool text = TEXT && jl >= GS_TEXT_MARK;
    bool settle = false;
    int np = pos;
    uint32_t c;
    if (text) {
        if (((jl >> 26) & 3u) != 3u)
            return gs_text_round<COUNT>(I, seq, iL, fwd, dir, l, u, jl, ju, pos, NSTOP, wb);
        /* text mode's LF step with base T[qs + d - 1]; J stays empty */
        c = (jl >> ((((jl >> 16) & 15u) - 1u) << 1)) & 3u;
    } else {
        settle = jpend;
        jpend = false;
        np = settle ? pos : pos + dir;
        if (np < 0 || np >= iL) return false;
        c = fwd ? gs_fwd_code(seq[np]) : gs_comp_code(seq[np]);
    }
    if (c > 3u) {
        if (!settle) {
            if (NSTOP) return false;
            pos = np;   /* wildcard: both intervals unchanged, so no new equality */
            return true;
        }
        /* settle over a wildcard: J unchanged */
    } else {
        uint32_t nl = l, nu = u;
        const bool had_j = jl <= ju;
        GsStepTouch touch;
        int blocks = gs_step_pair(I, nl, nu, jl, ju, c, !settle, touch);
        if (COUNT) wb += (unsigned long long)blocks;
        if (COUNT && wc) {
            wc->steps++;
            wc->lines256 += (unsigned long long)touch.lines256;
            wc->lines384 += (unsigned long long)touch.lines384;
            if (had_j) {
                wc->jsteps++;
                wc->jblocks += (unsigned long long)touch.jblocks;
                if (!settle && nl <= nu && nu - nl < u - l) wc->jshrank++;
            }
        }
        if (text) {
            l = nl;
            u = nu;
            const uint32_t d = ((jl >> 16) & 15u) - 1u;
            jl = (jl & ~(15u << 16)) | (d << 16);
            if (d) return true;
            if (!(jl & GS_TM_CONT)) return false;
            jl = 1u;
            ju = 0u;
            return true;
        }
        if (!settle) {
            if (nl > nu) return false;   /* natural end at pos */
            l = nl;
            u = nu;
            pos = np;
        }
    }
    if (jl <= ju && ju - jl == u - l) {
        killed = true;
        return false;
    }
    /* one row and no J: count the steps taken so (J's words are free);
     * after text_min of them the occurrence is no chance hit, and with 16
     * bases or more left the walker enters text mode */
    if (I.text_min && l == u && jl > ju) {
        if (jl < GS_REGIME_MARK) {
            jl = GS_REGIME_MARK;
            ju = 0u;
        } else if (++jl - GS_REGIME_MARK >= (uint32_t)I.text_min &&
                   (fwd ? pos : iL - 1 - pos) >= 16) {
            jl = GS_TEXT_MARK;
        }
    }
    return true;
}

/* A walk that found no room in the walker buffer: its start interval goes
 * to its own record slot under GS_LEFTOVER_MARK (no record has x = y = ~0),
 * and gs_search_leftover walks it after the other passes (its start and J
 * made again from the read). */
#define GS_LEFTOVER_MARK 0xffffffffu

__device__ __forceinline__ void gs_write_leftover(const GsBatch &B, uint32_t r, uint32_t n, bool fwd,
                                                  int anchor, uint32_t l, uint32_t u)
{
    const uint64_t slot = B.slot_off[r] + (fwd ? (uint64_t)(anchor - (B.k - 1))
                                               : (uint64_t)n + (uint64_t)anchor);
    if (slot < B.slot_cap) {
        GsRec rec;
        rec.x = (int32_t)GS_LEFTOVER_MARK;
        rec.y = (int32_t)GS_LEFTOVER_MARK;
        rec.l = l;
        rec.u = u;
        B.slots[slot] = rec;
        atomicOr(B.recmask + (slot >> 5), 1u << (slot & 31u));
        atomicOr(B.queue + 1, GS_FLAG_LEFTOVER);
    } else {
        atomicOr(B.queue + 1, GS_FLAG_OVERFLOW);
    }
}

/* per-warp reservation of walker-buffer entries: [next, end); full once a
 * reservation came back past the capacity (no further atomics, so the
 * 32-bit counter cannot wrap) */
struct GsReserve {
    uint32_t next, end, full;
};

template <int NSTOP, int COUNT>
__device__ __forceinline__ void gs_start_item(const GsDevIndex &I, const GsBatch &B, uint32_t r,
                                             uint32_t local, int lane, GsReserve &res,
                                             unsigned long long &wk, unsigned long long &wb)
{
    const uint32_t L = B.lengths[r];
    const int k = B.k;
    const uint32_t n = L - (uint32_t)k + 1u;
    const uint32_t nch = (n + GS_CHUNK - 1) / GS_CHUNK;
    const bool fwd = local < nch;
    const uint32_t chunk = fwd ? local : local - nch;
    const uint32_t ci = chunk * GS_CHUNK + (uint32_t)lane;
    const bool in_range = ci < n;
    /* lane 31 only starts the next item's first candidate (which that item
     * owns: ceil(n / GS_CHUNK) items cover every candidate) */
    const bool owned = in_range && lane < GS_CHUNK;
    const unsigned char *seq = (const unsigned char *)B.seqs + B.offsets[r];
    const int iL = (int)L;
    const int anchor = fwd ? (k - 1 + (int)ci) : ((int)n - 1 - (int)ci);
    const int dir = fwd ? -1 : 1;

    uint32_t l = 1, u = 0, fcode = 4;
    int pos = anchor;
    bool alive = false, ok = false, contained = false;
    if (in_range)
        ok = gs_start<NSTOP, false>(I, seq, anchor, dir, fwd, gs_start_len(I, k), iL, l, u, pos,
                                    alive, contained, fcode, wk, wb);
    /* lane+1 holds the neighbour toward the longer match (e+1 forward, s-1
     * reverse), started at far end pos - dir */
    const uint32_t nl = __shfl_down_sync(0xffffffffu, l, 1);
    const uint32_t nu = __shfl_down_sync(0xffffffffu, u, 1);
    const int nalive = __shfl_down_sync(0xffffffffu, alive ? 1 : 0, 1);

    bool killed = false, jpend = false;
    uint32_t jl = 1, ju = 0;
    if (owned && alive && ci + 1u < n) {
        const int nb = anchor - dir;
        const uint32_t cn = fwd ? gs_fwd_code(seq[nb]) : gs_comp_code(seq[nb]);
        if (cn <= 3u) {
            if (fcode < 4u) {
                killed = (fcode == cn);   /* otherwise X·cn does not occur: no J */
            } else if (nalive) {
                jl = nl;
                ju = nu;
                jpend = true;
            }
        }
        /* cn not ACGT: the candidates to the right never started; this one
         * walks without J and, if the rule would have stopped it, its record
         * is one the filters drop */
    }

    const bool walker = owned && alive && !killed;
    const uint32_t wm = __ballot_sync(0xffffffffu, walker);
    if (owned && !walker) gs_write_record(B, r, n, fwd, anchor, pos, l, u, ok, killed);
    if (!wm) return;
    /* entries for this item's walkers: the rest of the reservation, then a
     * new chunk */
    const uint32_t cnt = (uint32_t)__popc(wm);
    const uint32_t rank = (uint32_t)__popc(wm & ((1u << lane) - 1u));
    const uint32_t rem = res.end - res.next;
    uint32_t g = 0;
    if (rem < cnt) {
        if (res.full) {
            g = (uint32_t)B.walker_cap;
        } else {
            if (lane == 0) g = atomicAdd(B.queue + 2, gs_walker_chunk(B));
            g = __shfl_sync(0xffffffffu, g, 0);
            if ((uint64_t)g + gs_walker_chunk(B) >= B.walker_cap) res.full = 1u;
        }
    }
    if (walker) {
        uint64_t idx;
        if (rank < rem) idx = res.next + rank;
        else idx = (uint64_t)g + (rank - rem);
        const uint64_t cap_end = rank < rem ? res.end : min((uint64_t)g + gs_walker_chunk(B), B.walker_cap);
        /* the entry keeps 30 bits of anchor: reads of 2^30 bases or more
         * (none in practice) are left over too */
        if (idx < cap_end && iL < (1 << 30)) {
            GsWalker w;
            w.r = r;
            w.anchor = (uint32_t)anchor | (fwd ? GS_WALKER_FWD : 0u) | (jpend ? GS_WALKER_JPEND : 0u);
            w.l = l;
            w.u = u;
            w.jl = jl;
            w.ju = ju;
            B.walkers[idx] = w;
        } else {
            gs_write_leftover(B, r, n, fwd, anchor, l, u);
        }
    }
    if (rem < cnt) {
        res.next = (uint32_t)min((uint64_t)g + (cnt - rem), B.walker_cap);
        res.end = (uint32_t)min((uint64_t)g + gs_walker_chunk(B), B.walker_cap);
        if (res.next > res.end) res.next = res.end;
    } else {
        res.next += cnt;
    }
}

/* one walker-buffer entry of a warp's reservation (rank among the warp's
 * walkers of this item); false when the buffer is full (or the read too
 * long for the entry's anchor bits): the walk is then left over */
__device__ __forceinline__ bool gs_push_walker(const GsBatch &B, const GsReserve &res, uint32_t g,
                                               uint32_t rem, uint32_t rank, uint32_t r, bool fwd,
                                               int anchor, uint32_t l, uint32_t u, uint32_t jl,
                                               uint32_t ju, bool jpend, int iL)
{
    uint64_t idx;
    if (rank < rem) idx = res.next + rank;
    else idx = (uint64_t)g + (rank - rem);
    const uint64_t cap_end = rank < rem ? res.end : min((uint64_t)g + gs_walker_chunk(B), B.walker_cap);
    if (idx >= cap_end || iL >= (1 << 30)) return false;
    GsWalker w;
    w.r = r;
    w.anchor = (uint32_t)anchor | (fwd ? GS_WALKER_FWD : 0u) | (jpend ? GS_WALKER_JPEND : 0u);
    w.l = l;
    w.u = u;
    w.jl = jl;
    w.ju = ju;
    B.walkers[idx] = w;
    return true;
}

/* J of an owned candidate from its neighbour's start, as in gs_start_item:
 * a forced code settles containment, otherwise the neighbour's interval is
 * J one base short (jpend) */
__device__ __forceinline__ void gs_start_j(uint32_t cn, uint32_t fcode, bool nalive, uint32_t nl,
                                           uint32_t nu, bool &killed, bool &jpend, uint32_t &jl,
                                           uint32_t &ju)
{
    if (cn > 3u) return;
    if (fcode < 4u) {
        killed = (fcode == cn);
    } else if (nalive) {
        jl = nl;
        ju = nu;
        jpend = true;
    }
}

/* A paired work item: the windows s = GS_PCHUNK*local - 1 + lane of read r
 * (lanes 1..GS_PCHUNK own theirs; lanes 0 and 31 start their windows only
 * for the neighbours' J), each window's forward candidate (ending at
 * s+KT-1, neighbour e+1 = lane+1) and reverse candidate (starting at s,
 * neighbour s-1 = lane-1) from one start-table entry.  Records, J and
 * walkers are those of gs_start_item for each candidate. */
template <int NSTOP, int COUNT>
__device__ __forceinline__ void gs_start_pair_item(const GsDevIndex &I, const GsBatch &B, uint32_t r,
                                                   uint32_t local, int lane, GsReserve &res,
                                                   unsigned long long &wk, unsigned long long &wb)
{
    const int iL = (int)B.lengths[r];
    const int k = B.k, KT = I.kx;
    const uint32_t n = (uint32_t)(iL - k + 1);   /* candidates per strand (the item exists: L >= k) */
    const int s = (int)(local * GS_PCHUNK) - 1 + lane;
    const bool in_range = s >= 0 && s <= iL - KT;
    const bool owned = in_range && lane >= 1 && lane <= GS_PCHUNK;
    const bool vf = in_range && s >= k - KT;   /* forward candidate s+KT-1 >= k-1 */
    const bool vr = in_range && s <= iL - k;   /* reverse candidate s <= L-k */
    const unsigned char *seq = (const unsigned char *)B.seqs + B.offsets[r];
    const int ef = s + KT - 1;
    GsStart F, R;
    gs_start_pair<NSTOP>(I, seq, s, KT, iL, vf, vr, F, R, wk, wb);
    const uint32_t fnl = __shfl_down_sync(0xffffffffu, F.l, 1);
    const uint32_t fnu = __shfl_down_sync(0xffffffffu, F.u, 1);
    const int fna = __shfl_down_sync(0xffffffffu, F.alive ? 1 : 0, 1);
    const uint32_t rnl = __shfl_up_sync(0xffffffffu, R.l, 1);
    const uint32_t rnu = __shfl_up_sync(0xffffffffu, R.u, 1);
    const int rna = __shfl_up_sync(0xffffffffu, R.alive ? 1 : 0, 1);

    bool fk = false, fj = false, rk = false, rj = false;
    uint32_t fjl = 1, fju = 0, rjl = 1, rju = 0;
    if (owned && vf && F.alive && ef + 1 < iL)
        gs_start_j(gs_fwd_code(seq[ef + 1]), F.fcode, fna != 0, fnl, fnu, fk, fj, fjl, fju);
    if (owned && vr && R.alive && s >= 1)
        gs_start_j(gs_comp_code(seq[s - 1]), R.fcode, rna != 0, rnl, rnu, rk, rj, rjl, rju);

    const bool wf = owned && vf && F.alive && !fk;
    const bool wr = owned && vr && R.alive && !rk;
    if (owned && vf && !wf) gs_write_record(B, r, n, true, ef, F.pos, F.l, F.u, F.ok, fk);
    if (owned && vr && !wr) gs_write_record(B, r, n, false, s, R.pos, R.l, R.u, R.ok, rk);
    const uint32_t mf = __ballot_sync(0xffffffffu, wf), mr = __ballot_sync(0xffffffffu, wr);
    if (!(mf | mr)) return;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t cnt = (uint32_t)(__popc(mf) + __popc(mr));
    const uint32_t rem = res.end - res.next;
    uint32_t g = 0;
    if (rem < cnt) {
        if (res.full) {
            g = (uint32_t)B.walker_cap;
        } else {
            if (lane == 0) g = atomicAdd(B.queue + 2, gs_walker_chunk(B));
            g = __shfl_sync(0xffffffffu, g, 0);
            if ((uint64_t)g + gs_walker_chunk(B) >= B.walker_cap) res.full = 1u;
        }
    }
    if (wf && !gs_push_walker(B, res, g, rem, (uint32_t)__popc(mf & lt), r, true, ef, F.l, F.u,
                              fjl, fju, fj, iL))
        gs_write_leftover(B, r, n, true, ef, F.l, F.u);
    if (wr && !gs_push_walker(B, res, g, rem, (uint32_t)(__popc(mf) + __popc(mr & lt)), r, false,
                              s, R.l, R.u, rjl, rju, rj, iL))
        gs_write_leftover(B, r, n, false, s, R.l, R.u);
    if (rem < cnt) {
        res.next = (uint32_t)min((uint64_t)g + (cnt - rem), B.walker_cap);
        res.end = (uint32_t)min((uint64_t)g + gs_walker_chunk(B), B.walker_cap);
        if (res.next > res.end) res.next = res.end;
    } else {
        res.next += cnt;
    }
}

/* 5 CTAs of 256 per SM (48 registers, no spills): more lookups in flight
 * than 4 or 3 (config-3 search 101.1 / 101.8 / 104.5 ms) */
template <int NSTOP, int COUNT, bool PAIRED>
__global__ void __launch_bounds__(256, 5) gs_search_start(GsDevIndex I, GsBatch B, int queue_chunk)
{
    const int lane = threadIdx.x & 31;
    unsigned long long wk = 0, wb = 0;
    GsReserve res = {0u, 0u, B.walker_cap == 0 ? 1u : 0u};
    const uint32_t n_items = B.item_off[B.n_reads];
    for (;;) {
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(B.queue, (uint32_t)queue_chunk);
        first = __shfl_sync(0xffffffffu, first, 0);
        if (first >= n_items) break;
        uint32_t last = min(first + (uint32_t)queue_chunk, n_items);
        uint32_t lo = 0, hi = B.n_reads;
        while (lo + 1 < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (B.item_off[mid] <= first) lo = mid; else hi = mid;
        }
        uint32_t r = lo;
        for (uint32_t it = first; it < last; it++) {
            while (B.item_off[r + 1] <= it) r++;
            if (PAIRED) gs_start_pair_item<NSTOP, COUNT>(I, B, r, it - B.item_off[r], lane, res, wk, wb);
            else gs_start_item<NSTOP, COUNT>(I, B, r, it - B.item_off[r], lane, res, wk, wb);
        }
    }
    /* unused entries of the last reservation: holes */
    for (uint32_t i = res.next + (uint32_t)lane; i < res.end; i += 32) B.walkers[i].r = GS_WALKER_HOLE;
    if (COUNT) gs_add_work(B, wk, wb);
}

template <int NSTOP, int COUNT>
__global__ void __launch_bounds__(128, 8) gs_search_walk(GsDevIndex I, GsBatch B, uint32_t wsz)
{
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    unsigned long long wb = 0;
    /* walker indices fit 32 bits: the buffer holds at most 2^31 entries */
    uint32_t n_w = *(volatile uint32_t *)(B.queue + 2);
    if (n_w > B.walker_cap) n_w = (uint32_t)B.walker_cap;
    uint32_t win = 0, win_end = 0;   /* warp-uniform window of walker indices */
    bool have = false, exhausted = false, killed = false, jpend = false;
    bool tfull = B.text_cap == 0;   /* warp-uniform: the text-job buffer is full */
    uint32_t r = 0, l = 0, u = 0, jl = 0, ju = 0, n = 0;
    int anchor = 0, pos = 0, iL = 0, dir = 0;
    bool fwd = false;
    const unsigned char *seq = NULL;
    GsWalkCounts wc = {0ull, 0ull, 0ull, 0ull, 0ull, 0ull, 0ull};
    for (;;) {
        uint32_t need = __ballot_sync(0xffffffffu, !have);
        while (need && !exhausted) {
            if (win == win_end) {
                uint32_t g = 0;
                if (lane == 0) g = atomicAdd(B.queue + 3, wsz);
                g = __shfl_sync(0xffffffffu, g, 0);
                if (g >= n_w) {
                    exhausted = true;
                    break;
                }
                win = g;
                win_end = min(g + wsz, n_w);
            }
            const uint32_t take = min((uint32_t)__popc(need), win_end - win);
            const uint32_t rank = __popc(need & lt);
            if (((need >> lane) & 1u) && rank < take) {
                GsWalker w = B.walkers[win + rank];
                if (w.r != GS_WALKER_HOLE) {
                    r = w.r;
                    fwd = (w.anchor & GS_WALKER_FWD) != 0;
                    anchor = (int)(w.anchor & (GS_WALKER_JPEND - 1u));
                    dir = fwd ? -1 : 1;
                    pos = anchor + dir * (gs_start_len(I, B.k) - 1);
                    l = w.l;
                    u = w.u;
                    jl = w.jl;
                    ju = w.ju;
                    dir = fwd ? -1 : 1;
                    const uint32_t Lr = B.lengths[r];
                    iL = (int)Lr;
                    n = Lr - (uint32_t)B.k + 1u;
                    seq = (const unsigned char *)B.seqs + B.offsets[r];
                    have = true;
                    killed = false;
                    jpend = (w.anchor & GS_WALKER_JPEND) != 0;
                    if (COUNT && (jpend || jl <= ju)) wc.jwalkers++;
                }
            }
            win += take;
            need = __ballot_sync(0xffffffffu, !have);
        }
        if (!__ballot_sync(0xffffffffu, have)) {
            if (exhausted) break;
            continue;
        }
        if (have && !gs_walk_step<NSTOP, COUNT, false>(I, seq, iL, fwd, dir, l, u, jl, ju, pos,
                                                       jpend, killed, wb, &wc)) {
            gs_write_record(B, r, n, fwd, anchor, pos, l, u, true, killed);
            have = false;
        }
        /* walkers that entered text mode go to the text pass, so that no
         * lane of this pass runs the compare; without room they walk on */
        const bool tx = have && jl >= GS_TEXT_MARK;
        const uint32_t tm = __ballot_sync(0xffffffffu, tx);
        if (tm) {
            uint32_t g = 0xffffffffu;
            if (!tfull) {
                const int lead = __ffs(tm) - 1;
                if (lane == lead) g = atomicAdd(B.queue + 4, (uint32_t)__popc(tm));
                g = __shfl_sync(0xffffffffu, g, lead);
                if ((uint64_t)g + __popc(tm) > B.text_cap) tfull = true;
            }
            const uint64_t idx = (uint64_t)g + __popc(tm & lt);
            if (tx) {
                if (g != 0xffffffffu && idx < B.text_cap) {
                    GsTextJob t;
                    t.r = r;
                    t.anchor = (uint32_t)anchor | (fwd ? GS_WALKER_FWD : 0u);
                    t.pos = (uint32_t)pos;
                    t.l = l;
                    B.text_jobs[idx] = t;
                    have = false;
                } else {
                    jl = 1u;
                    ju = 0u;
                }
            }
        }
    }
    if (COUNT) {
        gs_add_work(B, 0, wb);
        unsigned long long v[7] = {wc.steps, wc.jsteps, wc.jblocks, wc.jshrank, wc.jwalkers,
                                   wc.lines256, wc.lines384};
        for (int i = 0; i < 7; i++) {
            for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
            if (lane == 0) atomicAdd(&B.work[4 + i], v[i]);
        }
    }
}

/* Text pass: the walkers the walk pass handed over, one per thread, each
 * run to its end in text mode (and back in the interval walk after a
 * wildcard base). */
template <int NSTOP, int COUNT>
__global__ void __launch_bounds__(256) gs_search_text(GsDevIndex I, GsBatch B)
{
    uint64_t n_jobs = B.queue[4];
    if (n_jobs > B.text_cap) n_jobs = B.text_cap;
    unsigned long long wb = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_jobs; j += stride) {
        const GsTextJob t = B.text_jobs[j];
        const uint32_t r = t.r;
        const bool fwd = (t.anchor & GS_WALKER_FWD) != 0;
        const int anchor = (int)(t.anchor & ~GS_WALKER_FWD);
        const int dir = fwd ? -1 : 1;
        const uint32_t Lr = B.lengths[r];
        const int iL = (int)Lr;
        const unsigned char *seq = (const unsigned char *)B.seqs + B.offsets[r];
        int pos = (int)t.pos;
        uint32_t l = t.l, u = t.l, jl = GS_TEXT_MARK, ju = 0u;
        bool jpend = false, killed = false;
        while (gs_walk_step<NSTOP, COUNT, true>(I, seq, iL, fwd, dir, l, u, jl, ju, pos, jpend,
                                                killed, wb)) {
        }
        gs_write_record(B, r, Lr - (uint32_t)B.k + 1u, fwd, anchor, pos, l, u, true, killed);
    }
    if (COUNT) gs_add_work(B, 0, wb);
}

/* ------------------------------------------------------------------ */
/* plain search: one read per thread */

/* Leftover pass: the walks the start pass left in their record slots
 * (GS_LEFTOVER_MARK), a warp per read, each slot's walk on one lane, started
 * again with its J as the start pass would have made it; the slot gets the
 * walk's record, or loses its record bit.  Returns at once when the start
 * pass left none. */
template <int NSTOP, int COUNT>
__global__ void __launch_bounds__(256) gs_search_leftover(GsDevIndex I, GsBatch B)
{
    if (!(*(volatile uint32_t *)(B.queue + 1) & GS_FLAG_LEFTOVER)) return;
    const int lane = threadIdx.x & 31;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const int k = B.k, KT = gs_start_len(I, k);
    unsigned long long wk = 0, wb = 0;
    for (uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < B.n_reads; r += nwarps) {
        const uint64_t base = B.slot_off[r], end = B.slot_off[r + 1];
        if (end > B.slot_cap) continue;
        const uint32_t n = (uint32_t)((end - base) >> 1);
        const int iL = (int)B.lengths[r];
        const unsigned char *seq = (const unsigned char *)B.seqs + B.offsets[r];
        for (uint32_t j = (uint32_t)lane; j < 2u * n; j += 32) {
            const uint64_t slot = base + j;
            if (!((B.recmask[slot >> 5] >> (slot & 31u)) & 1u)) continue;
            const GsRec rec = B.slots[slot];
            if ((uint32_t)rec.x != GS_LEFTOVER_MARK || (uint32_t)rec.y != GS_LEFTOVER_MARK) continue;
            const bool fwd = j < n;
            /* slot j: forward e = k-1+j, reverse s = j-n (gs_write_record) */
            const int anchor = fwd ? k - 1 + (int)j : (int)(j - n);
            const int dir = fwd ? -1 : 1;
            /* the walker as the start pass made it: its start, and J from
             * the start of its neighbour toward the longer match (gs_start_item) */
            uint32_t l, u, fcode, jl = 1u, ju = 0u;
            int pos;
            bool alive, contained, jpend = false, killed = false;
            gs_start<NSTOP, false>(I, seq, anchor, dir, fwd, KT, iL, l, u, pos, alive, contained,
                                   fcode, wk, wb);
            const int nb = anchor - dir;
            if (alive && fcode >= 4u && nb >= 0 && nb < iL &&
                (fwd ? gs_fwd_code(seq[nb]) : gs_comp_code(seq[nb])) <= 3u) {
                uint32_t nl, nu, nfc;
                int npos;
                bool nalive, ncont;
                gs_start<NSTOP, false>(I, seq, nb, dir, fwd, KT, iL, nl, nu, npos, nalive, ncont,
                                       nfc, wk, wb);
                if (nalive) {
                    jl = nl;
                    ju = nu;
                    jpend = true;
                }
            }
            while (alive && gs_walk_step<NSTOP, COUNT, true>(I, seq, iL, fwd, dir, l, u, jl, ju, pos,
                                                             jpend, killed, wb)) {
            }
            /* no record: drop the slot's bit (gs_write_record leaves it) */
            atomicAnd(B.recmask + (slot >> 5), ~(1u << (slot & 31u)));
            gs_write_record(B, r, n, fwd, anchor, pos, l, u, true, killed);
        }
    }
    if (COUNT) gs_add_work(B, wk, wb);
}

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
            uint32_t fcode = 4;
            bool ok = gs_start<NSTOP, true>(I, seq, anchor, dir, fwd, KT, iL, l, u, pos, alive, contained,
                                            fcode, w_kmer, w_blk);
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
            if (rec.y != 0) {
                const uint64_t slot = B.slot_off[r] + (fwd ? (uint64_t)(anchor - (k - 1))
                                                           : (uint64_t)n + (uint64_t)anchor);
                slots[slot - B.slot_off[r]] = rec;
                atomicOr(B.recmask + (slot >> 5), 1u << (slot & 31u));
            }
        }
    }
    if (B.work) {
        atomicAdd(&B.work[0], w_kmer);
        atomicAdd(&B.work[1], w_blk);
    }
}

/* ------------------------------------------------------------------ */

static int gs_launch_batched(const GsDevIndex &I, GsBatch &B, int queue_chunk, int ctas_per_sm,
                            uint32_t n_items, cudaStream_t st)
{
    int dev = 0, sms = 0;
    GS_CUDA(cudaGetDevice(&dev));
    GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (queue_chunk <= 0) queue_chunk = GS_QUEUE_CHUNK;
    const bool cnt = B.work != NULL, nstop = B.n_mode == GS_N_STOP;
    void (*start)(GsDevIndex, GsBatch, int) =
        B.paired ? (nstop ? (cnt ? gs_search_start<1, 1, true> : gs_search_start<1, 0, true>)
                          : (cnt ? gs_search_start<0, 1, true> : gs_search_start<0, 0, true>))
                 : (nstop ? (cnt ? gs_search_start<1, 1, false> : gs_search_start<1, 0, false>)
                          : (cnt ? gs_search_start<0, 1, false> : gs_search_start<0, 0, false>));
    void (*walk)(GsDevIndex, GsBatch, uint32_t) =
        nstop ? (cnt ? gs_search_walk<1, 1> : gs_search_walk<1, 0>)
              : (cnt ? gs_search_walk<0, 1> : gs_search_walk<0, 0>);
    if (ctas_per_sm <= 0) {
        int occ = 0;
        GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, start, 256, 0));
        ctas_per_sm = occ > 0 ? occ : 1;
    }
    uint32_t grid = (uint32_t)sms * (uint32_t)ctas_per_sm;
    if (n_items) {
        uint32_t need = (n_items + (uint32_t)queue_chunk - 1) / (uint32_t)queue_chunk;
        if (need < grid * 8) grid = (need + 7) / 8;
    }
    if (grid == 0) grid = 1;
    GS_CUDA(cudaMemsetAsync(B.queue, 0, sizeof(uint32_t), st));
    GS_CUDA(cudaMemsetAsync(B.queue + 2, 0, 2 * sizeof(uint32_t), st));
    B.walker_chunk = gs_share_size(B.walker_cap, grid * 8u, 16u, GS_WALKER_CHUNK);
    start<<<grid, 256, 0, st>>>(I, B, queue_chunk);
    GS_CUDA(cudaGetLastError());
    if (B.walker_cap) {
        int wocc = 0;
        GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&wocc, walk, 128, 0));
        const uint32_t wgrid = (uint32_t)sms * (uint32_t)(wocc > 0 ? wocc : 4);
        /* the buffer's capacity stands for its walkers (the count is on the
         * device): about an eighth of a warp's share a window */
        walk<<<wgrid, 128, 0, st>>>(I, B, gs_share_size(B.walker_cap, wgrid * 4u, 8u, GS_WALK_WINDOW));
        GS_CUDA(cudaGetLastError());
        if (B.text_cap) {
            void (*text)(GsDevIndex, GsBatch) =
                nstop ? (cnt ? gs_search_text<1, 1> : gs_search_text<1, 0>)
                      : (cnt ? gs_search_text<0, 1> : gs_search_text<0, 0>);
            text<<<(uint32_t)sms * 8u, 256, 0, st>>>(I, B);
            GS_CUDA(cudaGetLastError());
        }
    }
    void (*leftover)(GsDevIndex, GsBatch) =
        nstop ? (cnt ? gs_search_leftover<1, 1> : gs_search_leftover<1, 0>)
              : (cnt ? gs_search_leftover<0, 1> : gs_search_leftover<0, 0>);
    leftover<<<(uint32_t)sms * 8u, 256, 0, st>>>(I, B);
    GS_CUDA(cudaGetLastError());
    return GS_OK;
}

int gs_launch_search(const GsDevIndex &I, GsBatch &B, int kernel, int queue_chunk, int ctas_per_sm,
                     uint32_t n_items, cudaStream_t st)
{
    if (B.n_reads == 0) return GS_OK;
    if (kernel == GS_KERNEL_BATCHED) return gs_launch_batched(I, B, queue_chunk, ctas_per_sm, n_items, st);
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
    /* count_work: instances that also count the lookups they execute */
    const bool cnt = B.work != NULL, nstop = B.n_mode == GS_N_STOP;
    void (*batched)(GsDevIndex, GsBatch, int) =
        nstop ? (cnt ? gs_search_lockstep<1, 1> : gs_search_lockstep<1, 0>)
              : (cnt ? gs_search_lockstep<0, 1> : gs_search_lockstep<0, 0>);
    void (*tail)(GsDevIndex, GsBatch) = nstop ? (cnt ? gs_search_tail<1, 1> : gs_search_tail<1, 0>)
                                              : (cnt ? gs_search_tail<0, 1> : gs_search_tail<0, 0>);
    if (ctas_per_sm <= 0) {
        int occ = 0;
        GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched, 256, 0));
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
    batched<<<grid, 256, 0, st>>>(I, B, queue_chunk);
    GS_CUDA(cudaGetLastError());
    if (B.cont) {
        int tocc = 0;
        GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tocc, tail, 256, 0));
        uint32_t tgrid = (uint32_t)sms * (uint32_t)(tocc > 0 ? tocc : 4);
        tail<<<tgrid, 256, 0, st>>>(I, B);
        GS_CUDA(cudaGetLastError());
    }
    return GS_OK;
}
