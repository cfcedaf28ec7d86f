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
#include "gs_fm.cuh"

#include <stdlib.h>
#include <string.h>

struct gs_index {
    int device;
    GsDevIndex dev;
    uint32_t *d_occ;
    uint32_t *d_sa;
    uint2 *d_kmer;
    uint4 *d_kmerx;
    uint32_t *d_saf, *d_text, *d_isa;
    size_t occ_bytes, sa_bytes, kmer_bytes, kmerx_bytes, text_bytes;
    float l2_hit_ratio;
    uint32_t gen;   /* bumped whenever device pointers change */
};

extern "C" int gs_index_set_kmer_len(gs_index *idx, int kx);
extern "C" int gs_index_set_text(gs_index *idx, int min_steps);

#define GS_SAF_UNSET 0xfffffffeu
#define GS_CHAIN_MAX (1u << 20)   /* LF steps one chain may take */

/* Every row lies on one chain of LF steps that starts at a sampled row: the
 * chain of sampled row i0 (text position s0) visits the rows of positions
 * s0-1, s0-2, ... and ends before the next sampled row or at the row of
 * position 0 (row primary, whose BWT symbol is $).  One thread per chain;
 * the chains together take seq_len+1 LF steps.  The row of position s has
 * BWT base T[s-1], so the same pass writes the text.  A chain that ends
 * at a sampled row checks that row's sample against its own position, so
 * the samples and the BWT are checked against each other.  stat: rows
 * visited, errors, and (steps << 32 | position) of the chain step that reaches row
 * primary+1 when that row is not sampled. */
__global__ void gs_text_chain_kernel(GsDevIndex I, uint32_t *saf, uint8_t *t8, uint32_t *isa,
                                     unsigned long long *stat)
{
    unsigned long long visited = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < I.n_sa; j += stride) {
        if (*(volatile unsigned long long *)&stat[1]) break;
        uint32_t row = (uint32_t)(j * I.sa_intv);
        uint32_t s = j == 0 ? I.seq_len : I.sa[j];
        for (uint32_t t = 0;; t++) {
            /* a consistent index ends every chain within seq_len+1 steps;
             * an inconsistent one may cycle: bounded, and the other chains
             * give up once one has failed */
            if (t > I.seq_len || t >= GS_CHAIN_MAX || s > I.seq_len || row > I.seq_len ||
                ((t & 4095u) == 4095u && *(volatile unsigned long long *)&stat[1])) {
                atomicAdd(&stat[1], 1ull);
                break;
            }
            saf[row] = s;
            visited++;
            if (s % GS_ISA_STEP == 0) isa[s / GS_ISA_STEP] = row;
            if (row == I.primary || s == 0) {
                if (row != I.primary || s != 0) atomicAdd(&stat[1], 1ull);
                break;
            }
            const uint32_t ka = row - (row > I.primary ? 1u : 0u);
            const GsBlk B = gs_load_block(I.occ, ka >> 6);
            const uint32_t c = gs_block_base(B, ka);
            t8[s - 1] = (uint8_t)c;
            row = gs_L2(I, c) + gs_occ_in_block(B, ka, c);
            s--;
            if (row % I.sa_intv == 0) {
                /* the next chain's sample must continue this one */
                if (row > I.seq_len || (row ? I.sa[row / I.sa_intv] : I.seq_len) != s)
                    atomicAdd(&stat[1], 1ull);
                break;
            }
            if (row == I.primary + 1u) stat[2] = ((unsigned long long)(t + 1) << 32) | s;
        }
    }
    for (int o = 16; o > 0; o >>= 1) visited += __shfl_xor_sync(0xffffffffu, visited, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&stat[0], visited);
}

/* 16 bases of t8 per text word, base i at bits 2*(i & 15) */
__global__ void gs_text_pack_kernel(const uint8_t *t8, uint32_t seq_len, uint32_t *text,
                                    uint64_t n_words)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_words; w += stride) {
        uint32_t v = 0;
        const uint64_t b = w * 16;
        for (uint32_t i = 0; i < 16; i++)
            if (b + i < seq_len) v |= ((uint32_t)t8[b + i] & 3u) << (2 * i);
        text[w] = v;
    }
}

/* rows the chains did not reach (a consistent index leaves none) */
__global__ void gs_text_unset_kernel(const uint32_t *saf, uint64_t n, unsigned long long *stat)
{
    unsigned long long cnt = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        cnt += saf[i] == GS_SAF_UNSET;
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&stat[1], cnt);
}

int gs_build_text(GsDevIndex &I, uint32_t *saf, uint32_t *text, uint32_t *isa, cudaStream_t st)
{
    const uint64_t n_rows = (uint64_t)I.seq_len + 1;
    const uint64_t n_words = ((uint64_t)I.seq_len + 15) / 16;
    uint8_t *t8 = NULL;
    unsigned long long *stat = NULL;
    cudaError_t e;
    if ((e = cudaMalloc(&t8, I.seq_len ? I.seq_len : 1)) != cudaSuccess)
        return gs_cuda_fail(e, "cudaMalloc(text build)");
    if ((e = cudaMalloc(&stat, 4 * sizeof(unsigned long long))) != cudaSuccess) {
        cudaFree(t8);
        return gs_cuda_fail(e, "cudaMalloc(text build)");
    }
    int rc = GS_OK;
    unsigned long long h[4] = {0, 0, 0, 0};
    if ((e = cudaMemsetAsync(stat, 0, 4 * sizeof(unsigned long long), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(saf, 0xfe, n_rows * 4, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(text, 0, (n_words + 2) * 4, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(isa, 0, ((uint64_t)I.seq_len / GS_ISA_STEP + 1) * 4, st)) !=
            cudaSuccess) {
        rc = gs_cuda_fail(e, "text build");
    } else {
        GsDevIndex D = I;
        const uint64_t chains = I.n_sa;
        uint32_t grid = (uint32_t)((chains + 255) / 256);
        if (grid > 152u * 64u) grid = 152u * 64u;
        gs_text_chain_kernel<<<grid ? grid : 1, 256, 0, st>>>(D, saf, t8, isa, stat);
        gs_text_pack_kernel<<<152 * 16, 256, 0, st>>>(t8, I.seq_len, text, n_words);
        gs_text_unset_kernel<<<152 * 16, 256, 0, st>>>(saf, n_rows, stat);
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = cudaMemcpyAsync(h, stat, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            rc = gs_cuda_fail(e, "text build");
    }
    cudaFree(t8);
    cudaFree(stat);
    if (rc) return rc;
    if (h[0] != n_rows || h[1] != 0) {
        gs_set_error("index does not describe one text: %llu of %llu rows reached, %llu errors",
                     h[0], (unsigned long long)n_rows, h[1]);
        return GS_EFORMAT;
    }
    const uint32_t minus1 = 0xffffffffu;
    GS_CUDA(cudaMemcpy(saf, &minus1, 4, cudaMemcpyHostToDevice));
    I.quirk_lo = (uint32_t)(h[2] & 0xffffffffu);
    I.quirk_n = (uint32_t)(h[2] >> 32);
    return GS_OK;
}

/* Longer start table by reference length: one table entry per distinct
 * kx-mer the text can hold (4^kx around seq_len) */
/* the 16 high (hi) or low bits of a word of 16 two-bit bases, first base
 * (bits 30-31) at bit 15 */
__device__ __forceinline__ uint32_t gs_slice16(uint32_t w, bool hi)
{
    uint32_t x = (hi ? w >> 1 : w) & 0x55555555u;
    x = (x | (x >> 1)) & 0x33333333u;
    x = (x | (x >> 2)) & 0x0f0f0f0fu;
    x = (x | (x >> 4)) & 0x00ff00ffu;
    return (x | (x >> 8)) & 0x0000ffffu;
}

/* The file's base words of each block (16 two-bit bases per word, first
 * base in the top bits, seed_gen.cu:52-58) become the bit-sliced words the
 * kernels read (gs_fm.cuh): H0, H1 = high bits of bases 0-31, 32-63, L0, L1
 * = low bits, base i at bit 31 - (i & 31).  The counts stay. */
__global__ void gs_bitslice_kernel(uint32_t *occ, uint64_t nblk)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblk; b += stride) {
        uint32_t *p = occ + b * GS_BLOCK_WORDS + 4;
        const uint32_t w0 = p[0], w1 = p[1], w2 = p[2], w3 = p[3];
        p[0] = (gs_slice16(w0, true) << 16) | gs_slice16(w1, true);
        p[1] = (gs_slice16(w2, true) << 16) | gs_slice16(w3, true);
        p[2] = (gs_slice16(w0, false) << 16) | gs_slice16(w1, false);
        p[3] = (gs_slice16(w2, false) << 16) | gs_slice16(w3, false);
    }
}

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
    GS_ON_DEVICE(device);
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
    gs_bitslice_kernel<<<152 * 8, 256>>>(idx->d_occ, nblk);
    if ((e = cudaGetLastError()) != cudaSuccess) {
        gs_index_free(idx);
        return gs_cuda_fail(e, "occurrence table layout");
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
    cudaFree(idx->d_saf);
    cudaFree(idx->d_text);
    cudaFree(idx->d_isa);
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
    out->device_bytes =
        idx->occ_bytes + idx->sa_bytes + idx->kmer_bytes + idx->kmerx_bytes + idx->text_bytes;
    out->kmer_len = idx->dev.kx ? idx->dev.kx : GS_K0;
    out->text_min = idx->d_saf ? (idx->dev.text_min ? idx->dev.text_min : -1) : 0;
    return GS_OK;
}

uint32_t gs_index_generation(const gs_index *idx) { return idx->gen; }

extern "C" int gs_index_text_table(const gs_index *idx, int which, uint64_t first, uint64_t count,
                                   uint32_t *out)
{
    if (!idx || !out || which < 0 || which > 2) return GS_EINVAL;
    if (!idx->d_saf) {
        gs_set_error("the index has no text structures");
        return GS_ESTATE;
    }
    const uint64_t n = which == 0   ? (uint64_t)idx->dev.seq_len + 1
                       : which == 1 ? ((uint64_t)idx->dev.seq_len + 15) / 16
                                    : (uint64_t)idx->dev.seq_len / GS_ISA_STEP + 1;
    if (first > n || count > n - first) {
        gs_set_error("text table range [%llu, +%llu) outside [0, %llu)", (unsigned long long)first,
                     (unsigned long long)count, (unsigned long long)n);
        return GS_EINVAL;
    }
    const uint32_t *src = which == 0 ? idx->d_saf : which == 1 ? idx->d_text : idx->d_isa;
    GS_ON_DEVICE(idx->device);
    GS_CUDA(cudaMemcpy(out, src + first, count * 4, cudaMemcpyDeviceToHost));
    return GS_OK;
}

static void drop_text(gs_index *idx)
{
    cudaFree(idx->d_saf);
    cudaFree(idx->d_text);
    cudaFree(idx->d_isa);
    idx->d_saf = idx->d_text = idx->d_isa = NULL;
    idx->text_bytes = 0;
    GsDevIndex &D = idx->dev;
    D.saf = D.text = D.isa = NULL;
    D.quirk_lo = D.quirk_n = 0;
    D.text_min = 0;
}

extern "C" int gs_index_set_text(gs_index *idx, int min_steps)
{
    if (!idx) return GS_EINVAL;
    GS_ON_DEVICE(idx->device);
    GS_CUDA(cudaDeviceSynchronize());
    idx->gen++;
    if (min_steps == 0) {
        drop_text(idx);
        return GS_OK;
    }
    GsDevIndex &D = idx->dev;
    if (!idx->d_saf) {
        if (D.seq_len >= GS_REGIME_MARK) {
            gs_set_error("text structures need seq_len below %u", GS_REGIME_MARK);
            return GS_EINVAL;
        }
        const size_t saf_b = ((size_t)D.seq_len + 1) * 4;
        const size_t text_b = (((size_t)D.seq_len + 15) / 16 + 2) * 4;
        const size_t isa_b = ((size_t)D.seq_len / GS_ISA_STEP + 1) * 4;
        cudaError_t e;
        if ((e = cudaMalloc(&idx->d_saf, saf_b)) != cudaSuccess ||
            (e = cudaMalloc(&idx->d_text, text_b)) != cudaSuccess ||
            (e = cudaMalloc(&idx->d_isa, isa_b)) != cudaSuccess) {
            drop_text(idx);
            return gs_cuda_fail(e, "cudaMalloc(text structures)");
        }
        GsDevIndex B = D;
        int rc = gs_build_text(B, idx->d_saf, idx->d_text, idx->d_isa, 0);
        if (rc) {
            drop_text(idx);
            return rc;
        }
        idx->text_bytes = saf_b + text_b + isa_b;
        D.saf = idx->d_saf;
        D.text = idx->d_text;
        D.isa = idx->d_isa;
        D.quirk_lo = B.quirk_lo;
        D.quirk_n = B.quirk_n;
    }
    D.text_min = min_steps > 0 ? min_steps : 0;
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
    GS_ON_DEVICE(idx->device);
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
    GS_ON_DEVICE(idx->device);
    GS_CUDA(cudaDeviceSynchronize());
    idx->gen++;
    if (idx->d_kmerx) {
        cudaFree(idx->d_kmerx);
        idx->d_kmerx = NULL;
        idx->kmerx_bytes = 0;
    }
    idx->dev.kmerx = NULL;
    idx->dev.kx = 0;
    if (kx == GS_K0) return GS_OK;
    size_t bytes = (size_t)16 << (2 * kx);
    uint4 *t = NULL;
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
