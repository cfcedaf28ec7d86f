/*
 * walk_forms.c -- test infrastructure: counts the steps of two ways to stop
 * a candidate's backward walk, with the oracle's FM primitives.
 *
 *   canonical: the containment-stopped walk.  Candidate e carries J, the
 *     interval of its neighbour's string R[p..e+1] at its own far end p, and
 *     stops at the first p with |I(R[p..e])| == |J| (J non-empty), or at its
 *     natural end (I empty, read end, non-ACGT base).
 *   monotone: I alone to its natural end, one containment check there (what
 *     a right-extension check allows, since containment, once true, stays
 *     true as p falls).  Its extra cost is the steps a contained candidate
 *     walks on after the canonical walk stopped it.
 *
 * Forward candidates start from the 13-mer R[e-12..e] (R[e] at bits 0-1);
 * reverse candidates run the same walk over the reverse complement, which is
 * the reference's right extension over complement codes.  Prints one JSON
 * line of totals.
 *
 * usage: walk_forms <index prefix> <reads, one per line> <k> <max reads>
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

static const or_index *IDX;
static uint32_t L2[5];

/* one backward step with base c; false when the interval empties */
static int bw(uint32_t *l, uint32_t *u, int c)
{
    uint32_t ol, ou;
    or_occ2(IDX, *l - 1, *u, c, &ol, &ou);
    *l = L2[c] + ol + 1;
    *u = L2[c] + ou;
    return *l <= *u;
}

static uint32_t size_of(uint32_t l, uint32_t u) { return l <= u ? u - l + 1 : 0; }

/* 13-mer key ending at e (code[e] at bits 0-1); -1 when a base is not ACGT */
static int64_t key13(const uint8_t *code, int e)
{
    uint32_t pat = 0;
    for (int j = 0; j < 13; j++) {
        if (code[e - j] > 3) return -1;
        pat |= (uint32_t)code[e - j] << (2 * j);
    }
    return pat;
}

/* steps I alone takes from far end p to its natural end */
static unsigned long long natural_steps(const uint8_t *code, int p, uint32_t l, uint32_t u)
{
    unsigned long long n = 0;
    while (p - 1 >= 0 && code[p - 1] <= 3) {
        n++;
        if (!bw(&l, &u, code[p - 1])) break;
        p--;
    }
    return n;
}

int main(int argc, char **argv)
{
    if (argc < 5) {
        fprintf(stderr, "usage: %s prefix reads.txt k max_reads\n", argv[0]);
        return 2;
    }
    or_index *idx;
    if (or_index_load(argv[1], &idx)) {
        fprintf(stderr, "cannot load %s\n", argv[1]);
        return 1;
    }
    IDX = idx;
    or_index_L2(idx, L2);
    uint32_t *tab = malloc(sizeof(uint32_t) * 2 * ((size_t)1 << 26));
    if (!tab || or_kmer_table(idx, 13, tab, 0)) return 1;
    const int k = atoi(argv[3]);
    const long max_reads = atol(argv[4]);
    FILE *f = fopen(argv[2], "r");
    if (!f) return 1;
    static char line[1 << 20];
    static uint8_t code[1 << 20];
    unsigned long long cand = 0, started = 0, with_j = 0, killed = 0, killed_at_start = 0;
    unsigned long long steps = 0, steps_j = 0, steps_no_j = 0, j_shrank = 0, extra = 0;
    long n_reads = 0;
    while (n_reads < max_reads && fgets(line, sizeof line, f)) {
        int L = (int)strlen(line);
        while (L && (line[L - 1] == '\n' || line[L - 1] == '\r')) L--;
        n_reads++;
        if (L < k) continue;
        for (int strand = 0; strand < 2; strand++) {
            for (int i = 0; i < L; i++) {
                int c;
                switch (line[i]) {
                case 'A': case 'a': c = 0; break;
                case 'C': case 'c': c = 1; break;
                case 'G': case 'g': c = 2; break;
                case 'T': case 't': c = 3; break;
                default: c = 4;
                }
                if (strand == 0) code[i] = (uint8_t)c;
                else code[L - 1 - i] = (uint8_t)(c > 3 ? 4 : 3 - c);
            }
            for (int e = k - 1; e < L; e++) {
                cand++;
                const int64_t pat = key13(code, e);
                if (pat < 0) continue;
                uint32_t l = tab[2 * pat], u = tab[2 * pat + 1];
                if (l > u) continue;
                started++;
                int p = e - 12;
                /* J: the neighbour's 13-mer, one step back to far end p */
                uint32_t jl = 1, ju = 0;
                const int64_t pn = e + 1 < L ? key13(code, e + 1) : -1;
                if (pn >= 0) {
                    jl = tab[2 * pn];
                    ju = tab[2 * pn + 1];
                    if (!(jl <= ju && code[p] <= 3 && bw(&jl, &ju, code[p]))) {
                        jl = 1;
                        ju = 0;
                    }
                }
                if (jl <= ju) with_j++;
                if (jl <= ju && size_of(jl, ju) == size_of(l, u)) {
                    killed++;
                    killed_at_start++;
                    extra += natural_steps(code, p, l, u);
                    continue;
                }
                while (p - 1 >= 0 && code[p - 1] <= 3) {
                    const int c = code[p - 1];
                    steps++;
                    const int has_j = jl <= ju;
                    if (has_j) steps_j++;
                    else steps_no_j++;
                    uint32_t nl = l, nu = u;
                    if (!bw(&nl, &nu, c)) break;
                    if (has_j) {
                        if (size_of(nl, nu) < size_of(l, u)) j_shrank++;
                        if (!bw(&jl, &ju, c)) {
                            jl = 1;
                            ju = 0;
                        }
                    }
                    l = nl;
                    u = nu;
                    p--;
                    if (jl <= ju && size_of(jl, ju) == size_of(l, u)) {
                        killed++;
                        extra += natural_steps(code, p, l, u);
                        break;
                    }
                }
            }
        }
    }
    printf("{\"reads\": %ld, \"candidates\": %llu, \"started\": %llu, \"with_j\": %llu, "
           "\"killed\": %llu, \"killed_at_start\": %llu, \"steps_canonical\": %llu, "
           "\"steps_with_j\": %llu, \"steps_without_j\": %llu, \"j_steps_i_shrank\": %llu, "
           "\"extra_steps_to_natural_end\": %llu}\n",
           n_reads, cand, started, with_j, killed, killed_at_start, steps, steps_j, steps_no_j,
           j_shrank, extra);
    free(tab);
    or_index_free(idx);
    return 0;
}
