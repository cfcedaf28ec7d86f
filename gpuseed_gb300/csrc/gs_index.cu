/*
 * gs_index.cu -- index files -> device-resident index.
 *
 * Reads the reference's index files (bwt_restore_bwt / bwt_restore_sa,
 * seed_gen.cu:2685-2736) with the same header checks, but reports failures as
 * GS_E* codes instead of exit(1) (:2692-2707, :2720-2724), and checks that
 * the .bwt holds every occurrence block seq_len needs (the reference does
 * not).  On the device the blocks are padded to whole 32-byte blocks so that
 * every lookup is a single aligned 256-bit load, the sampled SA gets its
 * sa[0] = -1 sentinel (:2711) and the 13-mer table is built in HBM
 * (:2888-2895).
 */
#include "gs_internal.h"

#include <stdlib.h>
#include <string.h>

struct gs_index {
    int device;
    GsDevIndex dev;
    uint32_t *d_occ;
    uint32_t *d_sa;
    uint2 *d_kmer;
    uint2 *d_kmerx;
    size_t occ_bytes, sa_bytes, kmer_bytes, kmerx_bytes;
    float l2_hit_ratio;
};

extern "C" int gs_index_set_kmer_len(gs_index *idx, int kx);

/* Longer start table by reference length: one table entry per distinct
 * kx-mer the text can hold (4^kx around seq_len) */
static int auto_kmer_len(uint32_t seq_len)
{
    if (seq_len > (1u << 30)) return 16;
    if (seq_len > (1u << 28)) return 15;
    if (seq_len > (1u << 26)) return 14;
    return GS_K0;
}

extern "C" void gs_index_free(gs_index *idx);

static uint64_t expected_words(uint32_t seq_len)
{
    uint64_t n_occ = ((uint64_t)seq_len + GS_OCC_INTERVAL - 1) / GS_OCC_INTERVAL + 1;
    return 4 * n_occ + ((uint64_t)seq_len + 15) / 16;
}

const GsDevIndex *gs_index_dev(const gs_index *idx) { return &idx->dev; }
int gs_index_device(const gs_index *idx) { return idx->device; }
float gs_index_l2_ratio(const gs_index *idx) { return idx->l2_hit_ratio; }
size_t gs_index_occ_bytes(const gs_index *idx) { return idx->occ_bytes; }

static int upload(uint32_t primary, const uint32_t L2_1to4[4], const uint32_t *bwt,
                  uint64_t bwt_words, uint32_t sa_intv, const uint32_t *samples,
                  uint64_t n_samples, int device, gs_index **out)
{
    *out = NULL;
    uint32_t seq_len = L2_1to4[3];
    if (seq_len == 0 || primary > seq_len || L2_1to4[0] > L2_1to4[1] || L2_1to4[1] > L2_1to4[2] ||
        L2_1to4[2] > L2_1to4[3]) {
        gs_set_error("index header inconsistent (seq_len=%u primary=%u)", seq_len, primary);
        return GS_EFORMAT;
    }
    if (bwt_words < expected_words(seq_len)) {
        gs_set_error(".bwt holds %llu words, %llu needed for seq_len %u",
                     (unsigned long long)bwt_words, (unsigned long long)expected_words(seq_len),
                     seq_len);
        return GS_EFORMAT;
    }
    if (sa_intv == 0) {
        gs_set_error(".sa has sa_intv 0");
        return GS_EFORMAT;
    }
    uint64_t n_sa = ((uint64_t)seq_len + sa_intv) / sa_intv;
    if (n_samples + 1 != n_sa) {
        gs_set_error(".sa holds %llu samples, %llu expected", (unsigned long long)n_samples,
                     (unsigned long long)(n_sa - 1));
        return GS_EFORMAT;
    }
    GS_CUDA(cudaSetDevice(device));
    gs_index *idx = (gs_index *)calloc(1, sizeof(gs_index));
    if (!idx) return GS_ENOMEM;
    idx->device = device;
    uint64_t nblk = (uint64_t)seq_len / GS_OCC_INTERVAL + 2;
    idx->occ_bytes = nblk * GS_BLOCK_WORDS * 4;
    idx->sa_bytes = n_sa * 4;
    idx->kmer_bytes = (size_t)8 << (2 * GS_K0);
    cudaError_t e;
    if ((e = cudaMalloc(&idx->d_occ, idx->occ_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&idx->d_sa, idx->sa_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&idx->d_kmer, idx->kmer_bytes)) != cudaSuccess) {
        gs_index_free(idx);
        return gs_cuda_fail(e, "cudaMalloc(index)");
    }
    uint64_t copy_words = bwt_words < nblk * GS_BLOCK_WORDS ? bwt_words : nblk * GS_BLOCK_WORDS;
    if ((e = cudaMemset(idx->d_occ, 0, idx->occ_bytes)) != cudaSuccess ||
        (e = cudaMemcpy(idx->d_occ, bwt, copy_words * 4, cudaMemcpyHostToDevice)) != cudaSuccess) {
        gs_index_free(idx);
        return gs_cuda_fail(e, "index upload");
    }
    uint32_t minus1 = 0xffffffffu;
    if ((e = cudaMemcpy(idx->d_sa, &minus1, 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (n_samples && (e = cudaMemcpy(idx->d_sa + 1, samples, n_samples * 4,
                                      cudaMemcpyHostToDevice)) != cudaSuccess)) {
        gs_index_free(idx);
        return gs_cuda_fail(e, "sa upload");
    }
    GsDevIndex &D = idx->dev;
    D.occ = idx->d_occ;
    D.sa = idx->d_sa;
    D.kmer = idx->d_kmer;
    D.primary = primary;
    D.seq_len = seq_len;
    D.sa_intv = sa_intv;
    D.n_sa = (uint32_t)n_sa;
    D.L2[0] = 0;
    for (int c = 0; c < 4; c++) D.L2[c + 1] = L2_1to4[c];
    int rc = gs_build_kmer_table(D, idx->d_kmer, 0);
    if (rc == GS_OK && (e = cudaDeviceSynchronize()) != cudaSuccess) rc = gs_cuda_fail(e, "kmer table");
    if (rc) {
        gs_index_free(idx);
        return rc;
    }
    /* the longer table is an accelerator: without room for it, run without */
    for (int kx = auto_kmer_len(seq_len); kx > GS_K0; kx--)
        if (gs_index_set_kmer_len(idx, kx) == GS_OK) break;
    cudaGetLastError();
    *out = idx;
    return GS_OK;
}

extern "C" int gs_index_from_host(uint32_t primary, const uint32_t L2_1to4[4], const uint32_t *bwt,
                                  uint64_t bwt_words, uint32_t sa_intv,
                                  const uint32_t *sa_samples, uint64_t n_samples, int device,
                                  gs_index **out)
{
    if (!out || !L2_1to4 || !bwt || (n_samples && !sa_samples)) {
        gs_set_error("gs_index_from_host: null argument");
        return GS_EINVAL;
    }
    return upload(primary, L2_1to4, bwt, bwt_words, sa_intv, sa_samples, n_samples, device, out);
}

static int read_file(const char *fn, uint8_t **buf, size_t *len)
{
    FILE *fp = fopen(fn, "rb");
    if (!fp) {
        gs_set_error("cannot open %s", fn);
        return GS_EIO;
    }
    fseek(fp, 0, SEEK_END);
    long n = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    if (n < 0) {
        fclose(fp);
        gs_set_error("cannot size %s", fn);
        return GS_EIO;
    }
    uint8_t *b = (uint8_t *)malloc((size_t)n + 4);
    if (!b) {
        fclose(fp);
        return GS_ENOMEM;
    }
    if (fread(b, 1, (size_t)n, fp) != (size_t)n) {
        fclose(fp);
        free(b);
        gs_set_error("short read on %s", fn);
        return GS_EIO;
    }
    fclose(fp);
    *buf = b;
    *len = (size_t)n;
    return GS_OK;
}

extern "C" int gs_index_load(const char *prefix, int device, gs_index **out)
{
    if (!prefix || !out) {
        gs_set_error("gs_index_load: null argument");
        return GS_EINVAL;
    }
    *out = NULL;
    size_t pl = strlen(prefix);
    char *fn = (char *)malloc(pl + 8);
    if (!fn) return GS_ENOMEM;
    memcpy(fn, prefix, pl);
    strcpy(fn + pl, ".bwt");
    uint8_t *bw = NULL, *sa = NULL;
    size_t bwn = 0, san = 0;
    int rc = read_file(fn, &bw, &bwn);
    if (rc == GS_OK) {
        strcpy(fn + pl, ".sa");
        rc = read_file(fn, &sa, &san);
    }
    free(fn);
    if (rc == GS_OK) {
        uint32_t hb[5], hs[7];
        if (bwn < 20 || (bwn - 20) % 4 || san < 28 || (san - 28) % 4) {
            gs_set_error("index files truncated (.bwt %zu bytes, .sa %zu bytes)", bwn, san);
            rc = GS_EFORMAT;
        } else {
            memcpy(hb, bw, 20);
            memcpy(hs, sa, 28);
            if (hs[0] != hb[0]) {
                gs_set_error("SA-BWT inconsistency: primary is not the same");
                rc = GS_EFORMAT;
            } else if (hs[6] != hb[4]) {
                gs_set_error("SA-BWT inconsistency: seq_len is not the same");
                rc = GS_EFORMAT;
            } else {
                rc = upload(hb[0], hb + 1, (const uint32_t *)(bw + 20), (bwn - 20) / 4, hs[5],
                            (const uint32_t *)(sa + 28), (san - 28) / 4, device, out);
            }
        }
    }
    free(bw);
    free(sa);
    return rc;
}

extern "C" void gs_index_free(gs_index *idx)
{
    if (!idx) return;
    cudaFree(idx->d_occ);
    cudaFree(idx->d_sa);
    cudaFree(idx->d_kmer);
    cudaFree(idx->d_kmerx);
    free(idx);
}

extern "C" int gs_index_get_info(const gs_index *idx, gs_index_info *out)
{
    if (!idx || !out) return GS_EINVAL;
    out->seq_len = idx->dev.seq_len;
    out->primary = idx->dev.primary;
    out->sa_intv = idx->dev.sa_intv;
    out->n_sa = idx->dev.n_sa;
    for (int c = 0; c < 5; c++) out->L2[c] = idx->dev.L2[c];
    out->device = idx->device;
    out->device_bytes = idx->occ_bytes + idx->sa_bytes + idx->kmer_bytes + idx->kmerx_bytes;
    out->kmer_len = idx->dev.kx ? idx->dev.kx : GS_K0;
    return GS_OK;
}

extern "C" int gs_index_kmer_table(const gs_index *idx, uint64_t first, uint64_t count,
                                   uint32_t *out)
{
    if (!idx || !out) return GS_EINVAL;
    uint64_t n = (uint64_t)1 << (2 * GS_K0);
    if (first > n || count > n - first) {
        gs_set_error("k-mer table range [%llu, +%llu) outside [0, %llu)", (unsigned long long)first,
                     (unsigned long long)count, (unsigned long long)n);
        return GS_EINVAL;
    }
    GS_CUDA(cudaSetDevice(idx->device));
    GS_CUDA(cudaMemcpy(out, idx->d_kmer + first, count * 8, cudaMemcpyDeviceToHost));
    return GS_OK;
}

extern "C" int gs_index_set_l2_window(gs_index *idx, float hit_ratio)
{
    if (!idx || hit_ratio < 0.f || hit_ratio > 1.f) return GS_EINVAL;
    idx->l2_hit_ratio = hit_ratio;
    return GS_OK;
}

extern "C" int gs_index_set_kmer_len(gs_index *idx, int kx)
{
    if (!idx || kx < GS_K0 || kx > 16) {
        gs_set_error("k-mer start table length %d outside [13, 16]", kx);
        return GS_EINVAL;
    }
    GS_CUDA(cudaSetDevice(idx->device));
    if (idx->d_kmerx) {
        cudaFree(idx->d_kmerx);
        idx->d_kmerx = NULL;
        idx->kmerx_bytes = 0;
    }
    idx->dev.kmerx = NULL;
    idx->dev.kx = 0;
    if (kx == GS_K0) return GS_OK;
    size_t bytes = (size_t)8 << (2 * kx);
    uint2 *t = NULL;
    cudaError_t e = cudaMalloc(&t, bytes);
    if (e != cudaSuccess) return gs_cuda_fail(e, "cudaMalloc(k-mer start table)");
    int rc = gs_build_kmerx_table(idx->dev, t, kx, 0);
    if (rc == GS_OK && (e = cudaDeviceSynchronize()) != cudaSuccess) rc = gs_cuda_fail(e, "k-mer table");
    if (rc) {
        cudaFree(t);
        return rc;
    }
    idx->d_kmerx = t;
    idx->kmerx_bytes = bytes;
    idx->dev.kmerx = t;
    idx->dev.kx = kx;
    return GS_OK;
}
