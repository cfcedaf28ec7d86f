/*
 * gs_fm.cuh -- FM-index primitives on the device.
 *
 * The occurrence table in HBM: one 32-byte block per 64 rows of the
 * $-removed BWT string, {count of A, C, G, T before the block, H0, H1, L0,
 * L1}.  The counts are the reference's checkpoints (seed_gen.cu:52-58); the
 * block's 64 bases are stored bit-sliced instead of as 2-bit fields: H0/H1
 * hold their high bits and L0/L1 their low bits, base i of the block at bit
 * 31 - (i & 31) of word i >> 5 of each.  The loader converts the file's
 * packed words (16 bases per word, first base in the top bits) once
 * (gs_index.cu).  The arithmetic is the reference's (seed_gen.cu:195-216
 * occ, :329-368 occ pair, :455-484 LF); the counting is our own: the bases
 * equal to c among the first n of a block are the set bits of
 * (H ^ ~c1) & (L ^ ~c0) in the top n bits, two popcounts per query.
 */
#ifndef GS_FM_CUH
#define GS_FM_CUH

#include "gs_internal.h"

struct GsBlk {
    uint32_t w[8];
};

/* one random read-only word with a 64-byte L2 fill (the default fills 128) */
__device__ __forceinline__ uint32_t gs_ld64(const uint32_t *p)
{
    uint32_t v;
    asm("ld.global.nc.L2::64B.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ GsBlk gs_load_block(const uint32_t *occ, uint32_t blk)
{
    GsBlk b;
    const uint32_t *p = occ + (size_t)blk * GS_BLOCK_WORDS;
    asm("ld.global.nc.L2::64B.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(b.w[0]), "=r"(b.w[1]), "=r"(b.w[2]), "=r"(b.w[3]), "=r"(b.w[4]), "=r"(b.w[5]),
          "=r"(b.w[6]), "=r"(b.w[7])
        : "l"(p));
    return b;
}

__device__ __forceinline__ uint32_t gs_sel4(uint32_t c, uint32_t a0, uint32_t a1, uint32_t a2,
                                            uint32_t a3)
{
    return c == 0 ? a0 : c == 1 ? a1 : c == 2 ? a2 : a3;
}

__device__ __forceinline__ uint32_t gs_L2(const GsDevIndex &I, uint32_t c)
{
    return gs_sel4(c, I.L2[0], I.L2[1], I.L2[2], I.L2[3]);
}

/* bit-sliced match words of a block for base c: bit 31 - (i & 31) of word
 * i >> 5 is set when base i of the block is c */
struct GsMatch {
    uint32_t cnt, m0, m1;
};

__device__ __forceinline__ GsMatch gs_match(uint32_t cnt, uint32_t h0, uint32_t h1, uint32_t l0,
                                            uint32_t l1, uint32_t c)
{
    const uint32_t hx = ((c >> 1) & 1u) - 1u;   /* ~0 when c's high bit is 0 */
    const uint32_t lx = (c & 1u) - 1u;
    GsMatch m;
    m.cnt = cnt;
    m.m0 = (h0 ^ hx) & (l0 ^ lx);
    m.m1 = (h1 ^ hx) & (l1 ^ lx);
    return m;
}

/* count of c in string positions [0, k] given k's block matched for c: the
 * set bits among the top (k & 63) + 1 bits of m0:m1 */
__device__ __forceinline__ uint32_t gs_occ_in_match(const GsMatch &m, uint32_t k)
{
    const uint32_t j = k & 63u;
    const uint32_t c0 = __popc(m.m0 >> (31u - ((j & 31u) | ((j >> 5) * 31u))));
    const uint32_t c1 = j >= 32u ? __popc(m.m1 >> (63u - j)) : 0u;
    return m.cnt + c0 + c1;
}

/* count of c in string positions [0, k] given k's block */
__device__ __forceinline__ uint32_t gs_occ_in_block(const GsBlk &b, uint32_t k, uint32_t c)
{
    return gs_occ_in_match(gs_match(gs_sel4(c, b.w[0], b.w[1], b.w[2], b.w[3]), b.w[4], b.w[5],
                                    b.w[6], b.w[7], c),
                           k);
}

/* base at string position k given k's block */
__device__ __forceinline__ uint32_t gs_block_base(const GsBlk &b, uint32_t k)
{
    const uint32_t sh = 31u - (k & 31u);
    const bool hi = (k & 32u) != 0;
    const uint32_t h = ((hi ? b.w[5] : b.w[4]) >> sh) & 1u;
    const uint32_t l = ((hi ? b.w[7] : b.w[6]) >> sh) & 1u;
    return (h << 1) | l;
}

/* One backward-search step with base c in [0,3]: [l,u] -> [l',u'].
 * Returns the number of 32-byte blocks read (0..2). */
__device__ __forceinline__ int gs_step(const GsDevIndex &I, uint32_t &l, uint32_t &u, uint32_t c)
{
    const bool lz = (l == 0);            /* occ(-1) = 0 */
    const bool uf = (u == I.seq_len);    /* occ(seq_len) = total */
    uint32_t la = l - 1u;
    la -= (la >= I.primary) ? 1u : 0u;
    uint32_t ua = u - ((u >= I.primary) ? 1u : 0u);
    uint32_t bl = la >> 6, bu = ua >> 6;
    uint32_t ol = 0, ou;
    int nb = 0;
    GsBlk B;
    if (!uf) {
        B = gs_load_block(I.occ, bu);
        ou = gs_occ_in_block(B, ua, c);
        nb = 1;
    } else {
        ou = gs_sel4(c, I.L2[1], I.L2[2], I.L2[3], I.L2[4]) - gs_L2(I, c);
    }
    if (!lz) {
        if (uf || bl != bu) {
            B = gs_load_block(I.occ, bl);
            nb++;
        }
        ol = gs_occ_in_block(B, la, c);
    }
    uint32_t base = gs_L2(I, c);
    l = base + ol + 1u;
    u = base + ou;
    return nb;
}

/* The part of a block one occurrence query with base c reads: the count
 * of c before the block and the four bit-slice words (a 4-byte and a
 * 16-byte load of the same 32-byte sector).  Their L2 fills are 64 bytes
 * (the block and its neighbour), not 128: config-3 search 101.25 -> 100.9
 * ms (256-byte fills: 101.5). */
struct GsHalf {
    uint32_t cnt, h0, h1, l0, l1;
};

__device__ __forceinline__ GsHalf gs_load_half(const uint32_t *occ, uint32_t blk, uint32_t c)
{
    GsHalf h;
    const uint32_t *p = occ + (size_t)blk * GS_BLOCK_WORDS;
    asm("ld.global.nc.L2::64B.u32 %0, [%1];" : "=r"(h.cnt) : "l"(p + c));
    asm("ld.global.nc.L2::64B.v4.u32 {%0,%1,%2,%3}, [%4];"
        : "=r"(h.h0), "=r"(h.h1), "=r"(h.l0), "=r"(h.l1)
        : "l"(p + 4));
    return h;
}

/* h = s ? a : h, word by word */
__device__ __forceinline__ void gs_half_take(GsHalf &h, bool s, const GsHalf &a)
{
    h.cnt = s ? a.cnt : h.cnt;
    h.h0 = s ? a.h0 : h.h0;
    h.h1 = s ? a.h1 : h.h1;
    h.l0 = s ? a.l0 : h.l0;
    h.l1 = s ? a.l1 : h.l1;
}

/* count of c in string positions [0, k] given k's block */
__device__ __forceinline__ uint32_t gs_occ_in_half(const GsHalf &b, uint32_t k, uint32_t c)
{
    return gs_occ_in_match(gs_match(b.cnt, b.h0, b.h1, b.l0, b.l1, c), k);
}

/* how many distinct values among those of a..d that are valid */
__device__ __forceinline__ int gs_distinct4(uint32_t a, bool va, uint32_t b, bool vb, uint32_t c,
                                            bool vc, uint32_t d, bool vd)
{
    return (int)va + (int)(vb && !(va && b == a)) + (int)(vc && !(va && c == a) && !(vb && c == b)) +
           (int)(vd && !(va && d == a) && !(vb && d == b) && !(vc && d == c));
}

/* What one step of gs_step_pair touched, for the work counters: blocks
 * loaded for J alone, and the distinct 128-byte lines its bounds fall in
 * with this layout (256 rows a line) and with a 64-byte block of 192 rows
 * (384 rows a line). */
struct GsStepTouch {
    int jblocks, lines256, lines384;
};

/* One backward step with base c of an interval I = [l,u] (only when doI)
 * and of a sub-interval J = [jl,ju] of it (jl > ju: none; left unchanged).  J's
 * bounds lie between I's, so their blocks are loaded only where they differ
 * from the blocks of I's bounds, and all loads are issued before any is
 * used.  Returns the number of 32-byte blocks loaded (0..4); jblocks gets
 * the number loaded for J alone. */
__device__ __forceinline__ int gs_step_pair(const GsDevIndex &I, uint32_t &l, uint32_t &u,
                                            uint32_t &jl, uint32_t &ju, uint32_t c, bool doI,
                                            GsStepTouch &touch)
{
    const uint32_t P = I.primary;
    const bool lz = (l == 0), uf = (u == I.seq_len);
    uint32_t la = l - 1u;
    la -= (la >= P) ? 1u : 0u;
    const uint32_t ua = u - ((u >= P) ? 1u : 0u);
    const bool jn = jl <= ju;
    const bool jlz = jn && jl == 0, juf = jn && ju == I.seq_len;
    uint32_t jla = jl - 1u;
    jla -= (jla >= P) ? 1u : 0u;
    const uint32_t jua = ju - ((ju >= P) ? 1u : 0u);
    const uint32_t bu = ua >> 6, bl = la >> 6, jbu = jua >> 6, jbl = jla >> 6;
    /* distinct blocks: H0 = bu, H1 = bl, H2 = jbu, H3 = jbl */
    const bool n0 = doI && !uf;
    const bool n1 = doI && !lz && !(n0 && bl == bu);
    const bool n2 = jn && !juf && !(n0 && jbu == bu) && !(n1 && jbu == bl);
    const bool n3 = jn && !jlz && !(n0 && jbl == bu) && !(n1 && jbl == bl) && !(n2 && jbl == jbu);
    GsHalf H0, H1, H2, H3;
    if (n0) H0 = gs_load_half(I.occ, bu, c);
    if (n1) H1 = gs_load_half(I.occ, bl, c);
    if (n2) H2 = gs_load_half(I.occ, jbu, c);
    if (n3) H3 = gs_load_half(I.occ, jbl, c);
    const uint32_t base = gs_L2(I, c);
    const uint32_t total = gs_sel4(c, I.L2[1], I.L2[2], I.L2[3], I.L2[4]) - base;
    const uint32_t ou = uf ? total : gs_occ_in_half(H0, ua, c);
    GsHalf X = H0;
    gs_half_take(X, n1, H1);
    const uint32_t ol = lz ? 0u : gs_occ_in_half(X, la, c);
    if (jn) {
        GsHalf Y = H1;
        gs_half_take(Y, n0 && jbu == bu, H0);
        gs_half_take(Y, n2, H2);
        const uint32_t jou = juf ? total : gs_occ_in_half(Y, jua, c);
        GsHalf Z = H2;
        gs_half_take(Z, n1 && jbl == bl, H1);
        gs_half_take(Z, n0 && jbl == bu, H0);
        gs_half_take(Z, n3, H3);
        const uint32_t jol = jlz ? 0u : gs_occ_in_half(Z, jla, c);
        jl = base + jol + 1u;
        ju = base + jou;
    }
    if (doI) {
        l = base + ol + 1u;
        u = base + ou;
    }
    const bool vu = doI && !uf, vl = doI && !lz, vju = jn && !juf, vjl = jn && !jlz;
    touch.jblocks = (int)n2 + (int)n3;
    touch.lines256 = gs_distinct4(ua >> 8, vu, la >> 8, vl, jua >> 8, vju, jla >> 8, vjl);
    touch.lines384 = gs_distinct4(ua / 384u, vu, la / 384u, vl, jua / 384u, vju, jla / 384u, vjl);
    return (int)n0 + (int)n1 + (int)n2 + (int)n3;
}

__device__ __forceinline__ int gs_step_pair(const GsDevIndex &I, uint32_t &l, uint32_t &u,
                                            uint32_t &jl, uint32_t &ju, uint32_t c, bool doI)
{
    GsStepTouch t;
    return gs_step_pair(I, l, u, jl, ju, c, doI, t);
}

/* LF of a BWT row (bwt_inv_psi_gpu, seed_gen.cu:455-484).  lf_mode
 * GS_LF_GPUSEED reproduces its return of 0 for row primary+1; GS_LF_BWA
 * computes LF there as bwa does (seed_gen.cu:448-453). */
__device__ __forceinline__ uint32_t gs_lf(const GsDevIndex &I, uint32_t k, int lf_mode)
{
    if (k == I.primary) return 0;
    uint32_t ka = k - ((k > I.primary) ? 1u : 0u);
    if (lf_mode == GS_LF_GPUSEED && ka == I.primary) return 0;
    GsBlk B = gs_load_block(I.occ, ka >> 6);
    uint32_t c = gs_block_base(B, ka);
    return gs_L2(I, c) + gs_occ_in_block(B, ka, c);
}

#endif
