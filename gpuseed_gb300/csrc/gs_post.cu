/*
 * gs_post.cu -- per-read filtering, ordering and the sampled-SA locate.
 *
 * Replaces, for one batch, the reference's compaction (DeviceSelect::Flagged,
 * seed_gen.cu:3400-3401), the SMEM/MEM filters and counts (:865-1251), the
 * segmented sorts by begin (:1233, :3570) and the expansion + locate kernels
 * (:555-724):
 *
 *   gs_finalize_count  lane per read (warp per long read): compacts the
 *                      read's candidate slots in place and counts the
 *                      seeds/positions the filters keep;
 *   (scan)             exclusive sums of those counts over reads;
 *   gs_finalize_emit   thread per read: merges the forward (ascending end)
 *                      and reverse (ascending start) records by begin --
 *                      equal begins keep forward first, as the reference's
 *                      stable sort does -- and writes the output seeds;
 *   gs_expand          position -> seed map;
 *   gs_locate          thread per position: LF walk to a sampled row.
 *
 * Filter rules on the per-strand record lists (ascending end / start):
 *   SMEM forward: keep a record unless the next one has the same begin
 *        (:1000-1006); reverse: keep unless the previous has the same end
 *        (:1013-1019).
 *   MEM  forward: drop a record whose next record has the same begin and the
 *        same interval size (:1114-1120); its positions are its rows minus the
 *        rows of that next same-begin record's interval (:933-953, :624-667);
 *        reverse: the same toward the previous record with the same end.
 */
#include "gs_fm.cuh"



__device__ __forceinline__ uint32_t gs_size(const GsRec &r) { return r.u - r.l + 1u; }

/* decision for forward record R whose next record (when has_next) is N */
__device__ __forceinline__ void gs_fwd_rule_v(const GsRec &R, const GsRec &N, bool has_next,
                                              int smem, uint32_t max_occ, bool &keep,
                                              uint32_t &cnt, uint32_t &xl, uint32_t &xu)
{
    const bool same = has_next && N.x == R.x;
    uint32_t sz = gs_size(R);
    xl = 1; xu = 0;
    if (smem) {
        keep = !same;
        cnt = sz;
    } else {
        uint32_t nsz = same ? gs_size(N) : 0u;
        keep = !(same && nsz == sz);
        cnt = sz - nsz;
        if (same) { xl = N.l; xu = N.u; }
    }
    if (max_occ && sz > max_occ) keep = false;
}

/* decision for forward record o of list F[0..nf) */
__device__ __forceinline__ void gs_fwd_rule(const GsRec *F, uint32_t nf, uint32_t o, int smem,
                                            uint32_t max_occ, bool &keep, uint32_t &cnt,
                                            uint32_t &xl, uint32_t &xu)
{
    GsRec N;
    N.l = 1; N.u = 0; N.x = 0; N.y = 0;
    if (o + 1 < nf) N = F[o + 1];
    gs_fwd_rule_v(F[o], N, o + 1 < nf, smem, max_occ, keep, cnt, xl, xu);
}

/* decision for reverse record R whose previous record (when has_prev) is P */
__device__ __forceinline__ void gs_rev_rule_v(const GsRec &R, const GsRec &P, bool has_prev,
                                              int smem, uint32_t max_occ, bool &keep,
                                              uint32_t &cnt, uint32_t &xl, uint32_t &xu)
{
    const bool same = has_prev && P.y == R.y;
    uint32_t sz = gs_size(R);
    xl = 1; xu = 0;
    if (smem) {
        keep = !same;
        cnt = sz;
    } else {
        uint32_t psz = same ? gs_size(P) : 0u;
        keep = !(same && psz == sz);
        cnt = sz - psz;
        if (same) { xl = P.l; xu = P.u; }
    }
    if (max_occ && sz > max_occ) keep = false;
}

__device__ __forceinline__ void gs_rev_rule(const GsRec *Rv, uint32_t nr, uint32_t o, int smem,
                                            uint32_t max_occ, bool &keep, uint32_t &cnt,
                                            uint32_t &xl, uint32_t &xu)
{
    (void)nr;
    GsRec P;
    P.l = 1; P.u = 0; P.x = 0; P.y = 0;
    if (o > 0) P = Rv[o - 1];
    gs_rev_rule_v(Rv[o], P, o > 0, smem, max_occ, keep, cnt, xl, xu);
}

/* Compacts the records among slots s0..s0+n (flagged in the record mask;
 * the other slots were never written) to the front, in order; returns the
 * count.  Per 1024 slots: one round of mask words (a lane each, scanned
 * across the warp), then the records, 32 at a time -- lane j finds the j-th
 * set bit by binary lifting over the scan and __fns within its word.  A
 * record's target is never beyond its source, and a group's loads all come
 * before its writes, so compacting in place is safe. */
__device__ __forceinline__ uint32_t gs_warp_compact(GsRec *slots, const uint32_t *mask, uint64_t s0,
                                                    uint32_t n, int lane)
{
    uint32_t cnt = 0;
    if (n == 0) return 0;
    const uint64_t s1 = s0 + n;
    const uint64_t w0 = s0 >> 5, wend = (s1 + 31) >> 5;
    for (uint64_t wc = w0; wc < wend; wc += 32) {
        const uint64_t w = wc + (uint64_t)lane;
        uint32_t m = 0;
        if (w < wend) {
            m = mask[w];
            const uint64_t lo = w << 5;
            if (lo < s0) m &= 0xffffffffu << (uint32_t)(s0 - lo);
            if (lo + 32 > s1) m &= 0xffffffffu >> (uint32_t)(lo + 32 - s1);
        }
        const uint32_t c = __popc(m);
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        for (uint32_t g = 0; g < total; g += 32) {
            const uint32_t j = g + (uint32_t)lane;
            const uint32_t jj = j < total ? j : total - 1u;
            int L = 0;   /* first lane whose inclusive count exceeds jj */
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                uint32_t x = __shfl_sync(0xffffffffu, inc, L + step - 1);
                if (x <= jj) L += step;
            }
            const uint32_t word = __shfl_sync(0xffffffffu, m, L);
            const uint32_t before = __shfl_sync(0xffffffffu, inc - c, L);
            const uint32_t bit = __fns(word, 0, (int)(jj - before) + 1);
            GsRec rec;
            const bool v = j < total;
            if (v) rec = slots[((wc + (uint64_t)L) << 5) + bit];
            __syncwarp();
            if (v) slots[s0 + cnt + j] = rec;
            __syncwarp();
        }
        cnt += total;
    }
    return cnt;
}

/* Both strands of a read at once when their 2n slots fit one 1024-slot
 * round: forward records (slots s0..s0+n) go to s0 + rank, reverse ones
 * (s0+n..s0+2n) to s0 + n + rank -- one round of mask words, one of
 * records, for both.  Every target is at or before its source and earlier
 * records' targets lie before later records' sources, so in place is safe.
 * mine: lane j's record among the first 32 (forward, then reverse). */
__device__ __forceinline__ void gs_warp_compact_both(GsRec *slots, const uint32_t *mask, uint64_t s0,
                                                     uint32_t n, int lane, uint32_t &nf,
                                                     uint32_t &nr, GsRec &mine)
{
    const uint64_t s1 = s0 + n, s2 = s0 + 2ull * n;
    const uint64_t w0 = s0 >> 5, wend = (s2 + 31) >> 5;   /* at most 32 words */
    mine.x = mine.y = 0;
    mine.l = 1u;
    mine.u = 0u;
    const uint64_t w = w0 + (uint64_t)lane;
    uint32_t mf = 0, mr = 0;
    if (w < wend) {
        uint32_t m = mask[w];
        const uint64_t lo = w << 5;
        if (lo < s0) m &= 0xffffffffu << (uint32_t)(s0 - lo);
        if (lo + 32 > s2) m &= 0xffffffffu >> (uint32_t)(lo + 32 - s2);
        /* bits below s1 are forward slots */
        const uint32_t fmask = s1 <= lo ? 0u : (s1 >= lo + 32 ? 0xffffffffu
                                                              : ~(0xffffffffu << (uint32_t)(s1 - lo)));
        mf = m & fmask;
        mr = m & ~fmask;
    }
    const uint32_t cf = __popc(mf), cr = __popc(mr);
    uint32_t incf = cf, incr = cr;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t tf = __shfl_up_sync(0xffffffffu, incf, o);
        uint32_t tr = __shfl_up_sync(0xffffffffu, incr, o);
        if (lane >= o) {
            incf += tf;
            incr += tr;
        }
    }
    nf = __shfl_sync(0xffffffffu, incf, 31);
    nr = __shfl_sync(0xffffffffu, incr, 31);
    const uint32_t total = nf + nr;
    for (uint32_t g = 0; g < total; g += 32) {
        const uint32_t j = g + (uint32_t)lane;
        const bool v = j < total;
        const bool rev = j >= nf;
        const uint32_t jj = !v ? 0u : (rev ? j - nf : j);
        int L = 0;   /* first lane whose inclusive count (of this strand) exceeds jj */
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const uint32_t xf = __shfl_sync(0xffffffffu, incf, L + step - 1);
            const uint32_t xr = __shfl_sync(0xffffffffu, incr, L + step - 1);
            if ((rev ? xr : xf) <= jj) L += step;
        }
        const uint32_t wf = __shfl_sync(0xffffffffu, mf, L);
        const uint32_t wr = __shfl_sync(0xffffffffu, mr, L);
        const uint32_t bf = __shfl_sync(0xffffffffu, incf - cf, L);
        const uint32_t br = __shfl_sync(0xffffffffu, incr - cr, L);
        GsRec rec;
        rec.x = rec.y = 0;
        rec.l = 1u;
        rec.u = 0u;
        if (v) {
            const uint32_t word = rev ? wr : wf;
            const uint32_t bit = __fns(word, 0, (int)(jj - (rev ? br : bf)) + 1);
            rec = slots[((w0 + (uint64_t)L) << 5) + bit];
        }
        if (g == 0) mine = rec;
        __syncwarp();
        if (v) slots[(rev ? s1 : s0) + jj] = rec;
        __syncwarp();
    }
}

/* One strand of a read -- slots s0..s0+n -- compacted in place by one
 * thread: each flagged record moves to s0 + (its rank), in order, and the
 * rule decides it once its neighbour is known (forward: the next record,
 * one record behind; reverse: the previous one).  Adds the kept seeds and
 * their positions; returns the record count. */
__device__ __forceinline__ uint32_t gs_lane_compact(GsRec *slots, const uint32_t *mask, uint64_t s0,
                                                    uint32_t n, bool fwd, int smem,
                                                    uint32_t max_occ, uint64_t &seeds,
                                                    uint64_t &npos)
{
    const uint64_t s1 = s0 + n;
    uint32_t cnt = 0;
    GsRec prev;
    prev.x = prev.y = 0;
    prev.l = 1u;
    prev.u = 0u;
    bool keep;
    uint32_t c, xl, xu;
    for (uint64_t lo = s0 & ~31ull; lo < s1; lo += 32) {
        uint32_t m = mask[lo >> 5];
        if (lo < s0) m &= 0xffffffffu << (uint32_t)(s0 - lo);
        if (lo + 32 > s1) m &= 0xffffffffu >> (uint32_t)(lo + 32 - s1);
        while (m) {
            const uint32_t b = (uint32_t)__ffs(m) - 1u;
            m &= m - 1u;
            const GsRec rec = slots[lo + b];
            slots[s0 + cnt] = rec;   /* at or before its source: read already */
            if (fwd) {
                if (cnt) gs_fwd_rule_v(prev, rec, true, smem, max_occ, keep, c, xl, xu);
            } else {
                gs_rev_rule_v(rec, prev, cnt > 0, smem, max_occ, keep, c, xl, xu);
            }
            if ((!fwd || cnt) && keep && c) {
                seeds++;
                npos += c;
            }
            prev = rec;
            cnt++;
        }
    }
    if (fwd && cnt) {
        gs_fwd_rule_v(prev, prev, false, smem, max_occ, keep, c, xl, xu);
        if (keep && c) {
            seeds++;
            npos += c;
        }
    }
    return cnt;
}

/* reads whose two strands span at most this many slots are compacted by one
 * lane; longer ones by the whole warp */
#define GS_LANE_SLOTS 512u

/* a read compacted and counted by the whole warp (long reads) */
__device__ __noinline__ void gs_finalize_read_warp(const GsBatch &B, uint32_t r, uint64_t base,
                                                   uint64_t next, int lane)
{
    uint32_t n = (uint32_t)((next - base) >> 1);
    GsRec *F = B.slots + base;
    GsRec *Rv = F + n;
    uint32_t nf, nr;
    uint64_t seeds = 0, npos = 0;
    bool done = false;
    if (2u * n + 31u <= 1024u) {
        GsRec mine;
        gs_warp_compact_both(B.slots, B.recmask, base, n, lane, nf, nr, mine);
        if (nf + nr <= 32u) {
            /* lane j holds record j of [forward | reverse]: the rules'
             * neighbours are lanes j+1 (forward) and j-1 (reverse) */
            GsRec up, dn;
            up.x = __shfl_down_sync(0xffffffffu, mine.x, 1);
            up.y = __shfl_down_sync(0xffffffffu, mine.y, 1);
            up.l = __shfl_down_sync(0xffffffffu, mine.l, 1);
            up.u = __shfl_down_sync(0xffffffffu, mine.u, 1);
            dn.x = __shfl_up_sync(0xffffffffu, mine.x, 1);
            dn.y = __shfl_up_sync(0xffffffffu, mine.y, 1);
            dn.l = __shfl_up_sync(0xffffffffu, mine.l, 1);
            dn.u = __shfl_up_sync(0xffffffffu, mine.u, 1);
            const uint32_t j = (uint32_t)lane;
            bool keep = false;
            uint32_t cnt = 0, xl, xu;
            if (j < nf)
                gs_fwd_rule_v(mine, up, j + 1 < nf, B.smem, B.max_occ, keep, cnt, xl, xu);
            else if (j < nf + nr)
                gs_rev_rule_v(mine, dn, j > nf, B.smem, B.max_occ, keep, cnt, xl, xu);
            if (keep && cnt) {
                seeds = 1;
                npos = cnt;
            }
            done = true;
        }
    } else {
        nf = gs_warp_compact(B.slots, B.recmask, base, n, lane);
        nr = gs_warp_compact(B.slots, B.recmask, base + n, n, lane);
    }
    for (uint32_t o = lane; !done && o < nf; o += 32) {
        bool keep; uint32_t cnt, xl, xu;
        gs_fwd_rule(F, nf, o, B.smem, B.max_occ, keep, cnt, xl, xu);
        if (keep && cnt) { seeds++; npos += cnt; }
    }
    for (uint32_t o = lane; !done && o < nr; o += 32) {
        bool keep; uint32_t cnt, xl, xu;
        gs_rev_rule(Rv, nr, o, B.smem, B.max_occ, keep, cnt, xl, xu);
        if (keep && cnt) { seeds++; npos += cnt; }
    }
    for (int off = 16; off; off >>= 1) {
        seeds += __shfl_xor_sync(0xffffffffu, seeds, off);
        npos += __shfl_xor_sync(0xffffffffu, npos, off);
    }
    if (lane == 0) {
        B.rd_nf[r] = nf;
        B.rd_nr[r] = nr;
        B.rd_nseeds[r] = seeds;
        B.rd_npos[r] = npos;
    }
}

/* 32 consecutive reads per warp: a lane compacts and counts its own read
 * when it spans at most GS_LANE_SLOTS slots (few instructions a read, the
 * warp's loads spread over 32 reads); the warp then takes its longer reads
 * one at a time. */
__global__ void __launch_bounds__(256) gs_finalize_count(GsBatch B)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r0 = warp * 32u; r0 < B.n_reads; r0 += nwarps * 32u) {
        const uint32_t r = r0 + (uint32_t)lane;
        uint64_t base = 0, next = 0;
        bool longr = false;
        if (r < B.n_reads) {
            base = B.slot_off[r];
            next = B.slot_off[r + 1];
            if (next > B.slot_cap) {
                /* a replayed pass whose input needs more slots than it was
                 * sized for: nothing of this read is there; the host
                 * re-sizes */
                B.rd_nf[r] = 0;
                B.rd_nr[r] = 0;
                B.rd_nseeds[r] = 0;
                B.rd_npos[r] = 0;
                atomicOr(B.queue + 1, GS_FLAG_OVERFLOW);
            } else if (next - base > GS_LANE_SLOTS) {
                longr = true;
            } else {
                const uint32_t n = (uint32_t)((next - base) >> 1);
                uint64_t seeds = 0, npos = 0;
                const uint32_t nf = gs_lane_compact(B.slots, B.recmask, base, n, true, B.smem,
                                                    B.max_occ, seeds, npos);
                const uint32_t nr = gs_lane_compact(B.slots, B.recmask, base + n, n, false,
                                                    B.smem, B.max_occ, seeds, npos);
                B.rd_nf[r] = nf;
                B.rd_nr[r] = nr;
                B.rd_nseeds[r] = seeds;
                B.rd_npos[r] = npos;
            }
        }
        uint32_t lm = __ballot_sync(0xffffffffu, longr);
        while (lm) {
            const int src = __ffs(lm) - 1;
            lm &= lm - 1u;
            const uint64_t b0 = __shfl_sync(0xffffffffu, base, src);
            const uint64_t b1 = __shfl_sync(0xffffffffu, next, src);
            gs_finalize_read_warp(B, r0 + (uint32_t)src, b0, b1, lane);
        }
    }
}

__global__ void __launch_bounds__(128) gs_finalize_emit(GsBatch B, uint64_t *seed_pos)
{
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B.n_reads) return;
    uint64_t base = B.slot_off[r];
    uint32_t n = (uint32_t)((B.slot_off[r + 1] - base) >> 1);
    const GsRec *F = B.slots + base;
    const GsRec *Rv = F + n;
    uint32_t nf = B.rd_nf[r], nr = B.rd_nr[r];
    uint64_t s = B.seed_off[r];
    uint64_t p = B.pos_off[r];
    uint32_t a = 0, b = 0;
    /* each record loaded once: the forward list's current and next, the
     * reverse list's current and previous */
    GsRec none;
    none.x = none.y = 0;
    none.l = 1u;
    none.u = 0u;
    GsRec fc = nf ? F[0] : none, fn = nf > 1 ? F[1] : none;
    GsRec rc = nr ? Rv[0] : none, rp = none;
    while (a < nf || b < nr) {
        bool take_f;
        if (a >= nf) take_f = false;
        else if (b >= nr) take_f = true;
        else take_f = ((uint32_t)fc.x & 0x7fffffffu) <= ((uint32_t)rc.x & 0x7fffffffu);
        bool keep; uint32_t cnt, xl, xu;
        GsRec R;
        if (take_f) {
            gs_fwd_rule_v(fc, fn, a + 1 < nf, B.smem, B.max_occ, keep, cnt, xl, xu);
            R = fc;
            a++;
            fc = fn;
            fn = a + 1 < nf ? F[a + 1] : none;
        } else {
            gs_rev_rule_v(rc, rp, b > 0, B.smem, B.max_occ, keep, cnt, xl, xu);
            R = rc;
            b++;
            rp = rc;
            rc = b < nr ? Rv[b] : none;
        }
        if (keep && cnt) {
            if (s < B.seed_cap) {
                gs_seed_rec o;
                o.x = R.x; o.y = R.y; o.l = R.l; o.u = R.u;
                o.xl = xl; o.xu = xu; o.n_pos = cnt; o.pad = 0;
                B.seeds[s] = o;
                seed_pos[s] = p;
            }
            s++;
            p += cnt;
        }
    }
}

/* GS_MEM_NEXT_GPUSEED (MEM mode).  seeds_to_threads_mem (seed_gen.cu:635-650)
 * looks for a kept record's exclusion interval among the compacted records
 * that follow it (forward: same begin) or precede it (reverse: same end),
 * and its scan does not stop at the read's end, while the count kernel's
 * does (:927-989).  Inside the read the scan finds the filters' own
 * neighbour.  It leaves the read only from the read's last forward record
 * when the read has no reverse record -- into the next read that has
 * records, whose first record is then forward -- and from the read's first
 * reverse record when the read has no forward record, into the previous
 * read's last record.  The record it meets heads (ends) a run whose last
 * (first) record is kept, and a dropped record has the interval of the
 * record it was dropped for, so the interval found is that of the other
 * read's first forward (last reverse) output seed, when the begin (end)
 * matches.  The seed keeps its count and its rows become the first n_pos
 * rows from l outside that interval.  Thread per read, after the emit. */
__global__ void __launch_bounds__(128) gs_mem_next_kernel(GsBatch B)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B.n_reads) return;
    const uint64_t s0 = B.seed_off[r], s1 = B.seed_off[r + 1];
    if (s0 == s1 || s1 > B.seed_cap) return;
    uint64_t last_f = s1, first_r = s1;
    for (uint64_t s = s0; s < s1; s++) {
        if ((uint32_t)B.seeds[s].y >> 31) {
            if (first_r == s1) first_r = s;
        } else {
            last_f = s;
        }
    }
    if (last_f < s1 && first_r == s1) {
        /* the next read with seeds; its first seed in output order is
         * forward exactly when it has forward records */
        uint32_t q = r + 1;
        while (q < B.n_reads && B.seed_off[q + 1] == B.seed_off[q]) q++;
        if (q < B.n_reads && B.seed_off[q + 1] <= B.seed_cap) {
            for (uint64_t s = B.seed_off[q]; s < B.seed_off[q + 1]; s++) {
                const gs_seed_rec N = B.seeds[s];
                if ((uint32_t)N.y >> 31) continue;
                if (N.x == B.seeds[last_f].x) {
                    B.seeds[last_f].xl = N.l;
                    B.seeds[last_f].xu = N.u;
                }
                break;
            }
        }
    }
    if (first_r < s1 && last_f == s1 && r > 0) {
        uint32_t q = r - 1;
        while (q > 0 && B.seed_off[q + 1] == B.seed_off[q]) q--;
        if (B.seed_off[q + 1] > B.seed_off[q] && B.seed_off[q + 1] <= B.seed_cap) {
            for (uint64_t s = B.seed_off[q + 1]; s-- > B.seed_off[q];) {
                const gs_seed_rec P = B.seeds[s];
                if (!((uint32_t)P.y >> 31)) continue;
                if (P.y == B.seeds[first_r].y) {
                    B.seeds[first_r].xl = P.l;
                    B.seeds[first_r].xu = P.u;
                }
                break;
            }
        }
    }
}

__global__ void __launch_bounds__(256) gs_expand(const uint64_t *seed_pos, const gs_seed_rec *seeds,
                                                 const uint64_t *n_seeds_dev, uint64_t seed_cap,
                                                 uint32_t *pmap, uint64_t pos_cap)
{
    uint64_t n = *n_seeds_dev;
    if (n > seed_cap) n = seed_cap;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += stride) {
        uint64_t p = seed_pos[s];
        uint32_t cnt = seeds[s].n_pos;
        for (uint32_t i = 0; i < cnt && p + i < pos_cap; i++) pmap[p + i] = (uint32_t)s;
    }
}

__global__ void __launch_bounds__(256) gs_locate(GsDevIndex I, const gs_seed_rec *seeds,
                                                 const uint64_t *seed_pos, const uint32_t *pmap,
                                                 const uint64_t *n_pos_dev, uint64_t pos_cap,
                                                 uint32_t *out, int lf_mode, uint32_t *flags,
                                                 unsigned long long *work)
{
    uint64_t n_pos = *n_pos_dev;
    if (n_pos > pos_cap) n_pos = pos_cap;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    /* base is the same for every lane of a warp, so warps stay whole */
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n_pos; base += stride) {
        const uint64_t j = base + threadIdx.x;
        uint32_t steps = 0;
        const bool active = j < n_pos;
        if (active) {
            uint32_t s = pmap[j];
            gs_seed_rec S = seeds[s];
            /* the (j - first)-th row from l outside [xl, xu] */
            uint32_t row = S.l + (uint32_t)(j - seed_pos[s]);
            const uint32_t x0 = S.xl > S.l ? S.xl : S.l;
            if (S.xl <= S.xu && S.xu >= x0 && row >= x0) row += S.xu - x0 + 1u;
            /* locate_seeds_gpu (:668-684): LF until a sampled row; a
             * consistent index reaches one within seq_len+1 steps.  With
             * the full suffix array it is one read: the walk's result is
             * SA[row], except that the LF quirk sends the rows whose walk
             * passes row primary+1 to row 0, where sa[0] = -1 gives the
             * steps taken minus one -- position - quirk_lo. */
            const uint32_t cap = I.seq_len + 2u;
            bool bad = false;
            if (I.saf) {
                uint32_t v = gs_ld64(&I.saf[row]);
                if (lf_mode == GS_LF_GPUSEED && v - I.quirk_lo < I.quirk_n) v -= I.quirk_lo;
                out[j] = v;
            }
            while (!I.saf && row % I.sa_intv) {
                row = gs_lf(I, row, lf_mode);
                if (++steps > cap) {
                    bad = true;
                    break;
                }
            }
            if (bad) {
                atomicOr(flags, GS_FLAG_WALK);
                out[j] = 0xffffffffu;
            } else if (!I.saf) {
                out[j] = __ldg(&I.sa[row / I.sa_intv]) + steps;
            }
        }
        if (work) {
            unsigned long long st = steps, np = active ? 1ull : 0ull;
            for (int off = 16; off; off >>= 1) {
                st += __shfl_xor_sync(0xffffffffu, st, off);
                np += __shfl_xor_sync(0xffffffffu, np, off);
            }
            if ((threadIdx.x & 31) == 0 && np) {
                atomicAdd(&work[2], st);
                atomicAdd(&work[3], np);
            }
        }
    }
}

int gs_launch_finalize_count(const GsDevIndex &I, GsBatch &B, cudaStream_t st)
{
    (void)I;
    if (B.n_reads == 0) return GS_OK;
    uint32_t grid = (B.n_reads + 255) / 256;
    if (grid > 152u * 16u) grid = 152u * 16u;
    gs_finalize_count<<<grid, 256, 0, st>>>(B);
    GS_CUDA(cudaGetLastError());
    return GS_OK;
}

int gs_launch_finalize_emit(const GsDevIndex &I, GsBatch &B, cudaStream_t st)
{
    (void)I;
    if (B.n_reads == 0) return GS_OK;
    gs_finalize_emit<<<(B.n_reads + 127) / 128, 128, 0, st>>>(B, B.seed_pos);
    GS_CUDA(cudaGetLastError());
    if (!B.smem && B.mem_next == GS_MEM_NEXT_GPUSEED) {
        gs_mem_next_kernel<<<(B.n_reads + 127) / 128, 128, 0, st>>>(B);
        GS_CUDA(cudaGetLastError());
    }
    return GS_OK;
}

int gs_launch_locate(const GsDevIndex &I, GsBatch &B, uint64_t n_seeds, uint64_t n_pos,
                     cudaStream_t st)
{
    if (B.n_reads == 0 || B.seed_cap == 0 || B.pos_cap == 0) return GS_OK;
    uint64_t ns = n_seeds ? n_seeds : B.seed_cap;
    uint64_t np = n_pos ? n_pos : B.pos_cap;
    if (n_seeds == 0 && n_pos == 0) {
        /* totals known only on the device: persistent grids */
        ns = ns < 152ull * 256 * 32 ? ns : 152ull * 256 * 32;
        np = np < 152ull * 256 * 64 ? np : 152ull * 256 * 64;
    } else if (n_pos == 0 || n_seeds == 0) {
        return GS_OK;   /* nothing to locate */
    }
    gs_expand<<<(unsigned)((ns + 255) / 256), 256, 0, st>>>(B.seed_pos, B.seeds,
                                                             B.seed_off + B.n_reads, B.seed_cap,
                                                             B.pmap, B.pos_cap);
    GS_CUDA(cudaGetLastError());
    gs_locate<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(I, B.seeds, B.seed_pos, B.pmap,
                                                             B.pos_off + B.n_reads, B.pos_cap,
                                                             B.pos, B.lf_mode, B.queue + 1, B.work);
    GS_CUDA(cudaGetLastError());
    return GS_OK;
}
