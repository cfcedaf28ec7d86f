/*
 * gs_text.cu -- the text records of a result, formatted on the GPU.
 *
 * Same bytes as the reference's -o printing loop (seed_gen.cu:3625-3647) and
 * the host writer: per read a header line naming the mode and the read
 * number, then for every seed with positions "\nRead[b, e] -> " and its
 * positions as "+p" / "-p" joined by ", ", then "\n".
 *
 * The text is cut into tokens in output order -- per read a header, then per
 * seed its "Read[..] -> " part followed by one token per position, then the
 * read's closing newline.  With the per-read seed and position offsets every
 * token's index is a closed form:
 *   header of read r     2r + seed_off[r] + pos_off[r]
 *   seed s (of read r)   2r + 1 + s + seed_pos[s]
 *   position p (seed s)  2r + 2 + s + p
 *   end of read r        2r + 1 + seed_off[r+1] + pos_off[r+1]
 * so one kernel per token kind writes the token lengths, an exclusive scan
 * turns them into byte offsets, and the same kernels write the bytes.
 */
#include "gs_internal.h"

static __device__ const char k_h0[] = "/*===================================";
static __device__ const char k_h1[] = " seeds in read no. ";
static __device__ const char k_h2[] =
    " (Read[begin, End] -> starting position(s) on the reference)"
    "===================================*/\n";

__device__ __forceinline__ uint32_t gs_ndig(uint32_t v)
{
    uint32_t n = 1;
    uint64_t t = 10;
    while (n < 10 && v >= t) {
        n++;
        t *= 10;
    }
    return n;
}

/* decimal digits of v at p (nd = gs_ndig(v)); returns p + nd */
__device__ __forceinline__ char *gs_put_u32(char *p, uint32_t v, uint32_t nd)
{
    for (uint32_t i = nd; i > 0; i--) {
        p[i - 1] = (char)('0' + v % 10u);
        v /= 10u;
    }
    return p + nd;
}

__device__ __forceinline__ char *gs_put_str(char *p, const char *s, uint32_t n)
{
    for (uint32_t i = 0; i < n; i++) p[i] = s[i];
    return p + n;
}

__device__ __forceinline__ uint32_t gs_header_len(const GsTextArgs &a, uint32_t r)
{
    return (uint32_t)(sizeof(k_h0) - 1) + (a.smem ? 4u : 3u) + (uint32_t)(sizeof(k_h1) - 1) +
           gs_ndig(a.first_read_no + r) + (uint32_t)(sizeof(k_h2) - 1);
}

/* per read: the seed -> read map, header and end tokens */
template <int WRITE>
__global__ void gs_text_reads(GsTextArgs a)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.n_reads) return;
    const uint64_t s0 = a.seed_off[r], s1 = a.seed_off[r + 1];
    const uint64_t th = 2ull * r + s0 + a.pos_off[r];
    const uint64_t te = 2ull * r + 1ull + s1 + a.pos_off[r + 1];
    if (!WRITE) {
        for (uint64_t s = s0; s < s1; s++) a.sread[s] = r;
        a.off[th] = gs_header_len(a, r);
        a.off[te] = 1;
        return;
    }
    char *p = a.text + a.off[th];
    p = gs_put_str(p, k_h0, sizeof(k_h0) - 1);
    p = a.smem ? gs_put_str(p, "SMEM", 4) : gs_put_str(p, "MEM", 3);
    p = gs_put_str(p, k_h1, sizeof(k_h1) - 1);
    const uint32_t no = a.first_read_no + r;
    p = gs_put_u32(p, no, gs_ndig(no));
    gs_put_str(p, k_h2, sizeof(k_h2) - 1);
    a.text[a.off[te]] = '\n';
}

/* per seed with positions: "\nRead[b, e] -> " */
template <int WRITE>
__global__ void gs_text_seeds(GsTextArgs a)
{
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.n_seeds) return;
    const gs_seed_rec S = a.seeds[s];
    const uint64_t t = 2ull * a.sread[s] + 1ull + s + a.seed_pos[s];
    const uint32_t x = (uint32_t)S.x & 0x7fffffffu, y = (uint32_t)S.y & 0x7fffffffu;
    const uint32_t nx = gs_ndig(x), ny = gs_ndig(y);
    if (!WRITE) {
        a.off[t] = S.n_pos ? 13u + nx + ny : 0u;
        return;
    }
    if (!S.n_pos) return;
    char *p = a.text + a.off[t];
    p = gs_put_str(p, "\nRead[", 6);
    p = gs_put_u32(p, x, nx);
    p = gs_put_str(p, ", ", 2);
    p = gs_put_u32(p, y, ny);
    gs_put_str(p, "] -> ", 5);
}

/* per position: [", "] sign digits */
template <int WRITE>
__global__ void gs_text_positions(GsTextArgs a)
{
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n_pos) return;
    const uint32_t s = a.pmap[p];
    const uint64_t q = p - a.seed_pos[s];
    const uint64_t t = 2ull * a.sread[s] + 2ull + s + p;
    const uint32_t v = a.pos[p];
    const uint32_t nd = gs_ndig(v);
    if (!WRITE) {
        a.off[t] = (q ? 2u : 0u) + 1u + nd;
        return;
    }
    char *o = a.text + a.off[t];
    if (q) o = gs_put_str(o, ", ", 2);
    *o++ = ((uint32_t)a.seeds[s].y >> 31) ? '-' : '+';
    gs_put_u32(o, v, nd);
}

static int gs_text_pass(const GsTextArgs &a, bool write, cudaStream_t st)
{
    if (a.n_reads) {
        uint32_t g = (a.n_reads + 255) / 256;
        if (write) gs_text_reads<1><<<g, 256, 0, st>>>(a);
        else gs_text_reads<0><<<g, 256, 0, st>>>(a);
        GS_CUDA(cudaGetLastError());
    }
    if (a.n_seeds) {
        uint32_t g = (uint32_t)((a.n_seeds + 255) / 256);
        if (write) gs_text_seeds<1><<<g, 256, 0, st>>>(a);
        else gs_text_seeds<0><<<g, 256, 0, st>>>(a);
        GS_CUDA(cudaGetLastError());
    }
    if (a.n_pos) {
        uint32_t g = (uint32_t)((a.n_pos + 255) / 256);
        if (write) gs_text_positions<1><<<g, 256, 0, st>>>(a);
        else gs_text_positions<0><<<g, 256, 0, st>>>(a);
        GS_CUDA(cudaGetLastError());
    }
    return GS_OK;
}

int gs_launch_text_lengths(const GsTextArgs &a, cudaStream_t st)
{
    return gs_text_pass(a, false, st);
}

int gs_launch_text_write(const GsTextArgs &a, cudaStream_t st)
{
    return gs_text_pass(a, true, st);
}
