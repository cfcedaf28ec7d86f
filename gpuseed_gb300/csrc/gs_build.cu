/*
 * gs_build.cu -- index construction on the GPU.
 *
 * Replaces build_index.sh (bwa index -b sa -r R, then bwa index -b bwt with
 * OCC_INTERVAL 0x40; build_index.sh:36-75), whose bwa fork is not available:
 * it produces the .bwt/.sa pair in the layout the reference reads
 * (seed_gen.cu:2685-2736, :52-58) for a forward-strand text.
 *
 *   suffix array  prefix doubling (Manber-Myers) over dense 32-bit ranks:
 *                 initial keys pack the first 21 characters in base 5
 *                 ($ = 0 < A..T), every round sorts (rank[i], rank[i+h]) pairs
 *                 with a 64-bit LSD radix sort and re-ranks by a scan of
 *                 "key changed" flags, until all ranks are distinct;
 *   BWT           B[row] = T[SA[row]-1], the $ row dropped (primary);
 *   occurrences   per 64-row block: counts of A,C,G,T before the block
 *                 (scan of per-block counts) + 4 words of 16 bases, MSB
 *                 first;
 *   sampled SA    SA[i * sa_intv] for i >= 1.
 *
 * Memory: about 30 bytes per base on the device (keys and values double
 * buffered, ranks, flags); a 3.1 Gbp text needs ~95 GB of HBM.
 */
#include "gs_internal.h"

#include <cub/cub.cuh>

#include <stdlib.h>
#include <string.h>

static __global__ void init_keys21(const uint8_t *__restrict__ T, uint64_t n, uint64_t *keys,
                                   uint32_t *vals)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k = 0;
#pragma unroll
        for (int j = 0; j < 21; j++) {
            uint64_t p = i + (uint64_t)j;
            uint64_t c = p < n ? (uint64_t)T[p] + 1u : 0u;
            k = k * 5u + c;
        }
        keys[i] = k;
        vals[i] = (uint32_t)i;
    }
}

static __global__ void change_flags(const uint64_t *keys, uint64_t N, uint32_t *flags)
{
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N;
         j += (uint64_t)gridDim.x * blockDim.x)
        flags[j] = (j == 0 || keys[j] != keys[j - 1]) ? 1u : 0u;
}

static __global__ void scatter_ranks(const uint32_t *sa, const uint32_t *g, uint64_t N, uint32_t *rank)
{
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N;
         j += (uint64_t)gridDim.x * blockDim.x)
        rank[sa[j]] = g[j];
}

static __global__ void pair_keys(const uint32_t *rank, uint64_t n, uint64_t h, int b, uint64_t *keys,
                                 uint32_t *vals)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t hi = rank[i];
        uint64_t lo = (i + h <= n) ? rank[i + h] : 0u;
        keys[i] = (hi << b) | lo;
        vals[i] = (uint32_t)i;
    }
}

/* B[row] with the $ row marked 4; primary = row of suffix 0 */
static __global__ void bwt_rows(const uint8_t *T, const uint32_t *sa, uint64_t N, uint8_t *B,
                                uint32_t *primary)
{
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N;
         r += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t p = sa[r];
        if (p == 0) {
            B[r] = 4;
            *primary = (uint32_t)r;
        } else {
            B[r] = T[p - 1];
        }
    }
}

/* one thread per 64-row block of the $-removed string: 4 packed words and
 * the block's own base counts */
static __global__ void pack_blocks(const uint8_t *B, uint64_t n, uint32_t primary, uint32_t *occ,
                                   uint32_t *blkcnt, uint64_t nblk)
{
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblk;
         b += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t cnt[4] = {0, 0, 0, 0};
        uint32_t w[4] = {0, 0, 0, 0};
        for (int q = 0; q < 64; q++) {
            uint64_t s = b * 64 + (uint64_t)q;
            if (s >= n) break;
            uint64_t r = s + (s >= primary ? 1u : 0u);
            uint32_t c = B[r] & 3u;
            cnt[c]++;
            w[q >> 4] |= c << ((15 - (q & 15)) << 1);
        }
        for (int c = 0; c < 4; c++) blkcnt[(uint64_t)c * nblk + b] = cnt[c];
        uint32_t *o = occ + b * GS_BLOCK_WORDS;
        o[4] = w[0]; o[5] = w[1]; o[6] = w[2]; o[7] = w[3];
    }
}

static __global__ void write_counts(const uint32_t *scan, uint64_t nblk, uint32_t *occ)
{
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblk;
         b += (uint64_t)gridDim.x * blockDim.x)
        for (int c = 0; c < 4; c++) occ[b * GS_BLOCK_WORDS + c] = scan[(uint64_t)c * nblk + b];
}

static __global__ void gather_samples(const uint32_t *sa, uint64_t n_samples, uint32_t intv,
                                      uint32_t *out)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_samples;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = sa[(i + 1) * intv];
}

static unsigned grid_for(uint64_t n)
{
    uint64_t g = (n + 255) / 256;
    return (unsigned)(g > 152ull * 64 ? 152ull * 64 : (g ? g : 1));
}

struct DevMem {
    void *p[16];
    int n;
    DevMem() : n(0) {}
    ~DevMem()
    {
        for (int i = 0; i < n; i++) cudaFree(p[i]);
    }
    template <class T>
    cudaError_t alloc(T *&ptr, size_t count)
    {
        cudaError_t e = cudaMalloc(&ptr, count * sizeof(T) + 16);
        if (e == cudaSuccess) p[n++] = ptr;
        return e;
    }
    template <class T>
    void release(T *&ptr)
    {
        for (int i = 0; i < n; i++)
            if (p[i] == (void *)ptr) {
                cudaFree(ptr);
                p[i] = p[--n];
                ptr = NULL;
                return;
            }
    }
};

#define BCUDA(x)                                               \
    do {                                                       \
        cudaError_t _e = (x);                                  \
        if (_e != cudaSuccess) return gs_cuda_fail(_e, #x);    \
    } while (0)

/* Suffix array of T[0..n) + $ into d_sa (n+1 entries, device). */
static int build_sa(const uint8_t *d_T, uint64_t n, uint32_t *d_sa_out)
{
    DevMem m;
    const uint64_t N = n + 1;
    uint64_t *k0, *k1;
    uint32_t *v0, *v1, *rank;
    BCUDA(m.alloc(k0, N));
    BCUDA(m.alloc(k1, N));
    BCUDA(m.alloc(v0, N));
    BCUDA(m.alloc(v1, N));
    BCUDA(m.alloc(rank, N));
    int b = 1;
    while (b < 32 && (1ull << b) <= N + 1) b++;
    cub::DoubleBuffer<uint64_t> keys(k0, k1);
    cub::DoubleBuffer<uint32_t> vals(v0, v1);
    init_keys21<<<grid_for(N), 256>>>(d_T, n, keys.Current(), vals.Current());
    BCUDA(cudaGetLastError());
    size_t tmp_bytes = 0, scan_bytes = 0;
    BCUDA(cub::DeviceRadixSort::SortPairs(NULL, tmp_bytes, keys, vals, N, 0, 64));
    BCUDA(cub::DeviceScan::InclusiveSum(NULL, scan_bytes, v1, v1, N));
    uint8_t *tmp = NULL;
    size_t need = tmp_bytes > scan_bytes ? tmp_bytes : scan_bytes;
    BCUDA(m.alloc(tmp, need));
    int end_bit = 49;   /* 5^21 < 2^49 */
    uint64_t h = 21;
    for (int round = 0; round < 40; round++) {
        BCUDA(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, vals, N, 0, end_bit));
        uint32_t *g = vals.Alternate();
        change_flags<<<grid_for(N), 256>>>(keys.Current(), N, g);
        BCUDA(cudaGetLastError());
        BCUDA(cub::DeviceScan::InclusiveSum(tmp, scan_bytes, g, g, N));
        uint32_t groups = 0;
        BCUDA(cudaMemcpy(&groups, g + (N - 1), 4, cudaMemcpyDeviceToHost));
        if ((uint64_t)groups == N) {
            BCUDA(cudaMemcpy(d_sa_out, vals.Current(), N * 4, cudaMemcpyDeviceToDevice));
            return GS_OK;
        }
        scatter_ranks<<<grid_for(N), 256>>>(vals.Current(), g, N, rank);
        BCUDA(cudaGetLastError());
        pair_keys<<<grid_for(N), 256>>>(rank, n, h, b, keys.Current(), vals.Current());
        BCUDA(cudaGetLastError());
        end_bit = 2 * b;
        h *= 2;
    }
    gs_set_error("suffix sorting did not converge");
    return GS_EINVAL;
}

/* Builds the file-layout .bwt words and .sa samples on the host. */
static int build_arrays(const uint8_t *codes, uint64_t n, uint32_t sa_intv, uint32_t *primary_out,
                        uint32_t L2_out[4], uint32_t **bwt_out, uint64_t *bwt_words_out,
                        uint32_t **samples_out, uint64_t *n_samples_out)
{
    DevMem m;
    const uint64_t N = n + 1;
    uint8_t *d_T, *d_B;
    uint32_t *d_sa, *d_prim;
    BCUDA(m.alloc(d_T, n));
    BCUDA(cudaMemcpy(d_T, codes, n, cudaMemcpyHostToDevice));
    BCUDA(m.alloc(d_sa, N));
    {
        int rc = build_sa(d_T, n, d_sa);   /* its sort buffers are freed on return */
        if (rc) return rc;
    }
    DevMem m2;
    BCUDA(m2.alloc(d_B, N));
    BCUDA(m2.alloc(d_prim, 1));
    bwt_rows<<<grid_for(N), 256>>>(d_T, d_sa, N, d_B, d_prim);
    BCUDA(cudaGetLastError());
    uint32_t primary = 0;
    BCUDA(cudaMemcpy(&primary, d_prim, 4, cudaMemcpyDeviceToHost));
    uint64_t nblk = (n + 63) / 64;
    uint32_t *d_occ, *d_cnt;
    BCUDA(m2.alloc(d_occ, (nblk + 1) * GS_BLOCK_WORDS));
    BCUDA(m2.alloc(d_cnt, 4 * (nblk + 1)));
    BCUDA(cudaMemset(d_cnt, 0, 4 * (nblk + 1) * 4));
    pack_blocks<<<grid_for(nblk), 256>>>(d_B, n, primary, d_occ, d_cnt, nblk);
    BCUDA(cudaGetLastError());
    /* exclusive scans of the 4 per-block count rows; the extra slot of each
     * row is the total */
    uint32_t *d_scan;
    BCUDA(m2.alloc(d_scan, 4 * (nblk + 1)));
    size_t sb = 0;
    BCUDA(cub::DeviceScan::ExclusiveSum(NULL, sb, d_cnt, d_scan, nblk + 1));
    uint8_t *d_tmp;
    BCUDA(m2.alloc(d_tmp, sb + 16));
    uint32_t *d_rows;
    BCUDA(m2.alloc(d_rows, 4 * (nblk + 1)));
    for (int c = 0; c < 4; c++) {
        BCUDA(cudaMemcpy(d_rows + (uint64_t)c * (nblk + 1), d_cnt + (uint64_t)c * nblk, nblk * 4,
                         cudaMemcpyDeviceToDevice));
        BCUDA(cudaMemset(d_rows + (uint64_t)c * (nblk + 1) + nblk, 0, 4));
        BCUDA(cub::DeviceScan::ExclusiveSum(d_tmp, sb, d_rows + (uint64_t)c * (nblk + 1),
                                            d_scan + (uint64_t)c * (nblk + 1), nblk + 1));
    }
    /* re-stride the scans to the [c * nblk + b] layout write_counts reads */
    for (int c = 0; c < 4; c++)
        BCUDA(cudaMemcpy(d_cnt + (uint64_t)c * nblk, d_scan + (uint64_t)c * (nblk + 1), nblk * 4,
                         cudaMemcpyDeviceToDevice));
    write_counts<<<grid_for(nblk), 256>>>(d_cnt, nblk, d_occ);
    BCUDA(cudaGetLastError());
    uint32_t tot[4];
    for (int c = 0; c < 4; c++)
        BCUDA(cudaMemcpy(&tot[c], d_scan + (uint64_t)c * (nblk + 1) + nblk, 4, cudaMemcpyDeviceToHost));
    uint64_t n_samples = n / sa_intv;   /* rows intv, 2 intv, ... <= n */
    uint32_t *d_smp;
    BCUDA(m2.alloc(d_smp, n_samples + 1));
    if (n_samples) {
        gather_samples<<<grid_for(n_samples), 256>>>(d_sa, n_samples, sa_intv, d_smp);
        BCUDA(cudaGetLastError());
    }
    /* host: bwa's layout (whole blocks, the last block's used words, final
     * counts) */
    uint64_t words = 4 * (nblk + 1) + (n + 15) / 16;
    uint32_t *occ = (uint32_t *)malloc((nblk + 1) * GS_BLOCK_WORDS * 4);
    uint32_t *bwt = (uint32_t *)malloc(words * 4 + 16);
    uint32_t *smp = (uint32_t *)malloc(n_samples * 4 + 16);
    if (!occ || !bwt || !smp) {
        free(occ); free(bwt); free(smp);
        return GS_ENOMEM;
    }
    cudaError_t e = cudaMemcpy(occ, d_occ, nblk * GS_BLOCK_WORDS * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && n_samples) e = cudaMemcpy(smp, d_smp, n_samples * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        free(occ); free(bwt); free(smp);
        return gs_cuda_fail(e, "index download");
    }
    uint64_t k = 0;
    for (uint64_t bl = 0; bl < nblk; bl++) {
        const uint32_t *o = occ + bl * GS_BLOCK_WORDS;
        uint64_t rows = n - bl * 64 < 64 ? n - bl * 64 : 64;
        uint64_t nw = (rows + 15) / 16;
        memcpy(bwt + k, o, 16);
        memcpy(bwt + k + 4, o + 4, nw * 4);
        k += 4 + nw;
    }
    memcpy(bwt + k, tot, 16);
    k += 4;
    free(occ);
    uint32_t L2[4];
    L2[0] = tot[0];
    L2[1] = L2[0] + tot[1];
    L2[2] = L2[1] + tot[2];
    L2[3] = L2[2] + tot[3];
    *primary_out = primary;
    memcpy(L2_out, L2, 16);
    *bwt_out = bwt;
    *bwt_words_out = k;
    *samples_out = smp;
    *n_samples_out = n_samples;
    return GS_OK;
}

static int write_files(const char *prefix, uint32_t primary, const uint32_t L2[4], const uint32_t *bwt,
                       uint64_t words, uint32_t sa_intv, uint32_t seq_len, const uint32_t *smp,
                       uint64_t n_samples)
{
    size_t pl = strlen(prefix);
    char *fn = (char *)malloc(pl + 8);
    if (!fn) return GS_ENOMEM;
    memcpy(fn, prefix, pl);
    strcpy(fn + pl, ".bwt");
    FILE *fp = fopen(fn, "wb");
    int ok = fp != NULL;
    if (ok) {
        ok = fwrite(&primary, 4, 1, fp) == 1 && fwrite(L2, 4, 4, fp) == 4 &&
             fwrite(bwt, 4, words, fp) == words;
        ok = (fclose(fp) == 0) && ok;
    }
    if (ok) {
        strcpy(fn + pl, ".sa");
        fp = fopen(fn, "wb");
        ok = fp != NULL;
        if (ok) {
            ok = fwrite(&primary, 4, 1, fp) == 1 && fwrite(L2, 4, 4, fp) == 4 &&
                 fwrite(&sa_intv, 4, 1, fp) == 1 && fwrite(&seq_len, 4, 1, fp) == 1 &&
                 fwrite(smp, 4, n_samples, fp) == n_samples;
            ok = (fclose(fp) == 0) && ok;
        }
    }
    if (!ok) gs_set_error("cannot write %s", fn);
    free(fn);
    return ok ? GS_OK : GS_EIO;
}

int gs_index_from_host(uint32_t primary, const uint32_t L2_1to4[4], const uint32_t *bwt,
                       uint64_t bwt_words, uint32_t sa_intv, const uint32_t *sa_samples,
                       uint64_t n_samples, int device, gs_index **out);

extern "C" int gs_index_build(const uint8_t *codes, uint64_t n, uint32_t sa_intv, int device,
                              const char *prefix, gs_index **out)
{
    if (!codes || n == 0 || n >= 0xfffffffeull || sa_intv == 0 || (!prefix && !out)) {
        gs_set_error("gs_index_build: need 1 <= n < 2^32-1 codes, sa_intv > 0 and an output");
        return GS_EINVAL;
    }
    for (uint64_t i = 0; i < n; i++)
        if (codes[i] > 3) {
            gs_set_error("gs_index_build: code %u at %llu is not 0..3", codes[i], (unsigned long long)i);
            return GS_EINVAL;
        }
    GS_ON_DEVICE(device);
    uint32_t primary = 0, L2[4];
    uint32_t *bwt = NULL, *smp = NULL;
    uint64_t words = 0, n_samples = 0;
    int rc = build_arrays(codes, n, sa_intv, &primary, L2, &bwt, &words, &smp, &n_samples);
    if (rc == GS_OK && prefix)
        rc = write_files(prefix, primary, L2, bwt, words, sa_intv, (uint32_t)n, smp, n_samples);
    if (rc == GS_OK && out)
        rc = gs_index_from_host(primary, L2, bwt, words, sa_intv, smp, n_samples, device, out);
    free(bwt);
    free(smp);
    return rc;
}
