/*
 * gs_fm.cuh -- FM-index primitives on the device.
 *
 * One occurrence lookup = one 32-byte block = one 256-bit vector load
 * (ld.global.nc.v8.u32) of {4 checkpoint counts, 4 words of 2-bit BWT}.
 * The arithmetic is the reference's (seed_gen.cu:142-158 popcounts, :195-216
 * occ, :329-368 occ pair, :455-484 LF); the bit tricks are our own: a base
 * matches when its two bits XOR the replicated code are both zero, and the
 * bases after the queried row are removed with a mask instead of being
 * cleared and subtracted.
 */
#ifndef GS_FM_CUH
#define GS_FM_CUH

#include "gs_internal.h"

struct GsBlk {
    uint32_t w[8];
};

__device__ __forceinline__ GsBlk gs_load_block(const uint32_t *occ, uint32_t blk)
{
    GsBlk b;
    const uint32_t *p = occ + (size_t)blk * GS_BLOCK_WORDS;
    asm("ld.global.nc.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
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

/* lanes of w (2-bit bases) equal to c, as the even bit of each pair */
__device__ __forceinline__ uint32_t gs_match(uint32_t w, uint32_t c)
{
    uint32_t x = w ^ (c * 0x55555555u);
    return ~(x | (x >> 1)) & 0x55555555u;
}

/* count of c in string positions [0, k] given k's block */
__device__ __forceinline__ uint32_t gs_occ_in_block(const GsBlk &b, uint32_t k, uint32_t c)
{
    uint32_t kw = (k >> 4) & 3u;
    uint32_t tail = 0xffffffffu << ((15u - (k & 15u)) << 1);
    uint32_t m0 = kw > 0 ? 0xffffffffu : tail;
    uint32_t m1 = kw > 1 ? 0xffffffffu : (kw == 1 ? tail : 0u);
    uint32_t m2 = kw > 2 ? 0xffffffffu : (kw == 2 ? tail : 0u);
    uint32_t m3 = kw == 3 ? tail : 0u;
    uint32_t n = gs_sel4(c, b.w[0], b.w[1], b.w[2], b.w[3]);
    n += __popc(gs_match(b.w[4], c) & m0);
    n += __popc(gs_match(b.w[5], c) & m1);
    n += __popc(gs_match(b.w[6], c) & m2);
    n += __popc(gs_match(b.w[7], c) & m3);
    return n;
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
 * of c before the block and the four BWT words (a 4-byte and a 16-byte
 * load of the same 32-byte sector). */
struct GsHalf {
    uint32_t cnt, w4, w5, w6, w7;
};

__device__ __forceinline__ GsHalf gs_load_half(const uint32_t *occ, uint32_t blk, uint32_t c)
{
    GsHalf h;
    const uint32_t *p = occ + (size_t)blk * GS_BLOCK_WORDS;
    asm("ld.global.nc.u32 %0, [%1];" : "=r"(h.cnt) : "l"(p + c));
    asm("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];"
        : "=r"(h.w4), "=r"(h.w5), "=r"(h.w6), "=r"(h.w7)
        : "l"(p + 4));
    return h;
}

/* h = s ? a : h, word by word */
__device__ __forceinline__ void gs_half_take(GsHalf &h, bool s, const GsHalf &a)
{
    h.cnt = s ? a.cnt : h.cnt;
    h.w4 = s ? a.w4 : h.w4;
    h.w5 = s ? a.w5 : h.w5;
    h.w6 = s ? a.w6 : h.w6;
    h.w7 = s ? a.w7 : h.w7;
}

/* count of c in string positions [0, k] given k's block */
__device__ __forceinline__ uint32_t gs_occ_in_half(const GsHalf &b, uint32_t k, uint32_t c)
{
    uint32_t kw = (k >> 4) & 3u;
    uint32_t tail = 0xffffffffu << ((15u - (k & 15u)) << 1);
    uint32_t m0 = kw > 0 ? 0xffffffffu : tail;
    uint32_t m1 = kw > 1 ? 0xffffffffu : (kw == 1 ? tail : 0u);
    uint32_t m2 = kw > 2 ? 0xffffffffu : (kw == 2 ? tail : 0u);
    uint32_t m3 = kw == 3 ? tail : 0u;
    uint32_t n = b.cnt;
    n += __popc(gs_match(b.w4, c) & m0);
    n += __popc(gs_match(b.w5, c) & m1);
    n += __popc(gs_match(b.w6, c) & m2);
    n += __popc(gs_match(b.w7, c) & m3);
    return n;
}

/* One backward step with base c of an interval I = [l,u] (only when doI)
 * and of a sub-interval J = [jl,ju] of it (jl > ju: none; left unchanged).  J's
 * bounds lie between I's, so their blocks are loaded only where they differ
 * from the blocks of I's bounds, and all loads are issued before any is
 * used.  Returns the number of 32-byte blocks loaded (0..4). */
__device__ __forceinline__ int gs_step_pair(const GsDevIndex &I, uint32_t &l, uint32_t &u,
                                            uint32_t &jl, uint32_t &ju, uint32_t c, bool doI)
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
    return (int)n0 + (int)n1 + (int)n2 + (int)n3;
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
    uint32_t kw = (ka >> 4) & 3u;
    uint32_t word = gs_sel4(kw, B.w[4], B.w[5], B.w[6], B.w[7]);
    uint32_t c = (word >> ((~ka & 15u) << 1)) & 3u;
    return gs_L2(I, c) + gs_occ_in_block(B, ka, c);
}

#endif
