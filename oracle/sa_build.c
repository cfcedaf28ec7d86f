/*
 * sa_build.c -- suffix array (SA-IS) and .bwt/.sa writer for test fixtures.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  The product builds its indexes on
 * the GPU (gpuseed_gb300/csrc/gs_build.cu); this file is the independent CPU
 * construction the GPU builder is checked against.
 *
 * SA-IS follows the published algorithm of Nong, Zhang and Chan ("Two
 * efficient algorithms for linear time suffix array construction", IEEE
 * Trans. Computers 2011; DCC 2009): classify S/L types, induce-sort the LMS
 * substrings, name them, recurse when names repeat, and induce the final
 * order from the sorted LMS suffixes.
 *
 * The files follow the layout the reference reads (seed_gen.cu:2685-2736)
 * with its 64-row, 32-bit occurrence blocks (seed_gen.cu:29, :52-58), as the
 * un-vendored bwa fork writes them (build_index.sh:54-75).
 */
#include "oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define TGET(t, i) ((t)[(i) >> 3] >> ((i) & 7) & 1)
#define TSET(t, i, v) ((v) ? ((t)[(i) >> 3] |= (uint8_t)(1u << ((i) & 7))) \
                           : ((t)[(i) >> 3] &= (uint8_t)~(1u << ((i) & 7))))
#define IS_LMS(t, i) ((i) > 0 && TGET(t, i) && !TGET(t, (i) - 1))

/* s: int32 string of length n over [0, K), s[n-1] == 0 unique smallest.
 * Types: 1 = S, 0 = L. */
static void buckets(const int32_t *s, int64_t n, int64_t K, int64_t *bkt, int end)
{
    memset(bkt, 0, sizeof(int64_t) * (size_t)K);
    for (int64_t i = 0; i < n; i++) bkt[s[i]]++;
    int64_t sum = 0;
    for (int64_t c = 0; c < K; c++) {
        sum += bkt[c];
        bkt[c] = end ? sum : sum - bkt[c];
    }
}

static void induce(const int32_t *s, int32_t *SA, int64_t n, int64_t K, const uint8_t *t,
                   int64_t *bkt)
{
    buckets(s, n, K, bkt, 0);
    for (int64_t i = 0; i < n; i++) {
        int64_t j = (int64_t)SA[i] - 1;
        if (SA[i] > 0 && !TGET(t, j)) SA[bkt[s[j]]++] = (int32_t)j;
    }
    buckets(s, n, K, bkt, 1);
    for (int64_t i = n - 1; i >= 0; i--) {
        int64_t j = (int64_t)SA[i] - 1;
        if (SA[i] > 0 && TGET(t, j)) SA[--bkt[s[j]]] = (int32_t)j;
    }
}

static int sais(const int32_t *s, int32_t *SA, int64_t n, int64_t K)
{
    uint8_t *t = (uint8_t *)calloc((size_t)(n / 8 + 1), 1);
    int64_t *bkt = (int64_t *)malloc(sizeof(int64_t) * (size_t)K);
    if (!t || !bkt) { free(t); free(bkt); return -1; }
    TSET(t, n - 1, 1);
    if (n >= 2) TSET(t, n - 2, 0);
    for (int64_t i = n - 3; i >= 0; i--)
        TSET(t, i, (s[i] < s[i + 1] || (s[i] == s[i + 1] && TGET(t, i + 1))) ? 1 : 0);

    /* stage 1: sort LMS substrings */
    buckets(s, n, K, bkt, 1);
    for (int64_t i = 0; i < n; i++) SA[i] = -1;
    for (int64_t i = 1; i < n; i++)
        if (IS_LMS(t, i)) SA[--bkt[s[i]]] = (int32_t)i;
    induce(s, SA, n, K, t, bkt);

    /* compact the sorted LMS positions into SA[0..n1) */
    int64_t n1 = 0;
    for (int64_t i = 0; i < n; i++)
        if (IS_LMS(t, SA[i])) SA[n1++] = SA[i];
    for (int64_t i = n1; i < n; i++) SA[i] = -1;

    /* name the LMS substrings */
    int64_t name = 0, prev = -1;
    for (int64_t i = 0; i < n1; i++) {
        int64_t pos = SA[i];
        int diff = 0;
        for (int64_t d = 0; d < n; d++) {
            if (prev == -1 || s[pos + d] != s[prev + d] || TGET(t, pos + d) != TGET(t, prev + d)) {
                diff = 1;
                break;
            } else if (d > 0 && (IS_LMS(t, pos + d) || IS_LMS(t, prev + d))) {
                break;
            }
        }
        if (diff) { name++; prev = pos; }
        SA[n1 + pos / 2] = (int32_t)(name - 1);
    }
    for (int64_t i = n - 1, j = n - 1; i >= n1; i--)
        if (SA[i] >= 0) SA[j--] = SA[i];

    /* stage 2: order the LMS suffixes, recursing when names repeat */
    int32_t *SA1 = SA, *s1 = SA + n - n1;
    if (name < n1) {
        if (sais(s1, SA1, n1, name)) { free(t); free(bkt); return -1; }
    } else {
        for (int64_t i = 0; i < n1; i++) SA1[s1[i]] = (int32_t)i;
    }

    /* stage 3: induce the full order from the sorted LMS suffixes */
    buckets(s, n, K, bkt, 1);
    for (int64_t i = 1, j = 0; i < n; i++)
        if (IS_LMS(t, i)) s1[j++] = (int32_t)i;
    for (int64_t i = 0; i < n1; i++) SA1[i] = s1[SA1[i]];
    for (int64_t i = n1; i < n; i++) SA[i] = -1;
    for (int64_t i = n1 - 1; i >= 0; i--) {
        int32_t j = SA[i];
        SA[i] = -1;
        SA[--bkt[s[j]]] = j;
    }
    induce(s, SA, n, K, t, bkt);
    free(t);
    free(bkt);
    return 0;
}

int or_suffix_array(const uint8_t *codes, uint64_t n, uint32_t *sa_out)
{
    if (n + 1 > 0x7fffffffull) return -5;
    int32_t *s = (int32_t *)malloc(sizeof(int32_t) * (n + 1));
    int32_t *SA = (int32_t *)malloc(sizeof(int32_t) * (n + 1));
    if (!s || !SA) { free(s); free(SA); return -4; }
    for (uint64_t i = 0; i < n; i++) {
        if (codes[i] > 3) { free(s); free(SA); return -5; }
        s[i] = (int32_t)codes[i] + 1;
    }
    s[n] = 0;
    int rc = sais(s, SA, (int64_t)n + 1, 5);
    if (rc == 0)
        for (uint64_t i = 0; i <= n; i++) sa_out[i] = (uint32_t)SA[i];
    free(s);
    free(SA);
    return rc ? -4 : 0;
}

/* .bwt: primary, L2[1..4], then per 64 rows of the $-removed BWT string a
 * block of 4 cumulative counts followed by up to 4 words of 16 two-bit bases
 * (most significant first), and a final count block. */
int or_build_index(const uint8_t *codes, uint64_t n, uint32_t sa_intv, const char *prefix)
{
    if (n == 0 || n >= 0xffffffffull || sa_intv == 0) return -5;
    uint32_t *SA = (uint32_t *)malloc(sizeof(uint32_t) * (n + 1));
    if (!SA) return -4;
    int rc = or_suffix_array(codes, n, SA);
    if (rc) { free(SA); return rc; }

    uint32_t L2[5] = {0, 0, 0, 0, 0};
    for (uint64_t i = 0; i < n; i++) L2[codes[i] + 1]++;
    for (int c = 1; c <= 4; c++) L2[c] += L2[c - 1];
    uint32_t primary = 0;
    uint64_t nw = 4 * ((n + 63) / 64 + 1) + (n + 15) / 16;
    uint32_t *buf = (uint32_t *)calloc(nw, 4);
    if (!buf) { free(SA); return -4; }
    uint32_t cnt[4] = {0, 0, 0, 0};
    uint64_t k = 0, i = 0;
    uint32_t word = 0;
    for (uint64_t row = 0; row <= n; row++) {
        if (SA[row] == 0) { primary = (uint32_t)row; continue; }
        uint8_t c = codes[SA[row] - 1];
        if (i % 64 == 0) { memcpy(buf + k, cnt, 16); k += 4; }
        word |= (uint32_t)c << ((15 - (i & 15)) << 1);
        if ((i & 15) == 15) { buf[k++] = word; word = 0; }
        cnt[c]++;
        i++;
    }
    if (i & 15) buf[k++] = word;
    memcpy(buf + k, cnt, 16);
    k += 4;

    size_t pl = strlen(prefix);
    char *fn = (char *)malloc(pl + 8);
    if (!fn) { free(SA); free(buf); return -4; }
    memcpy(fn, prefix, pl);
    strcpy(fn + pl, ".bwt");
    FILE *fp = fopen(fn, "wb");
    if (!fp) { free(fn); free(SA); free(buf); return -2; }
    fwrite(&primary, 4, 1, fp);
    fwrite(L2 + 1, 4, 4, fp);
    fwrite(buf, 4, k, fp);
    fclose(fp);

    /* .sa: primary, L2[1..4], sa_intv, seq_len, SA[intv], SA[2 intv], ... */
    strcpy(fn + pl, ".sa");
    fp = fopen(fn, "wb");
    if (!fp) { free(fn); free(SA); free(buf); return -2; }
    uint32_t seq_len = (uint32_t)n;
    fwrite(&primary, 4, 1, fp);
    fwrite(L2 + 1, 4, 4, fp);
    fwrite(&sa_intv, 4, 1, fp);
    fwrite(&seq_len, 4, 1, fp);
    for (uint64_t row = sa_intv; row <= n; row += sa_intv) fwrite(&SA[row], 4, 1, fp);
    fclose(fp);
    free(fn);
    free(SA);
    free(buf);
    return 0;
}
