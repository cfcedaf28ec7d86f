/*
 * gs_tools.cu -- measurement probes (no counterpart in the reference).
 *
 * gs_probe_random_gather: the random-sector roofline of the seeding path.
 * Every occurrence lookup of the search is one 32-byte block at an
 * unpredictable address; this probe issues independent 32- or 64-byte
 * vector loads at uniformly random aligned addresses of a buffer larger than
 * L2 and reports the loaded bytes per second (CUDA events, after warm-up).
 */
#include "gs_internal.h"

static __device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

template <int WORDS>
static __global__ void __launch_bounds__(256) gather_kernel(const uint32_t *__restrict__ buf,
                                                            uint64_t n_blocks, uint64_t per_thread,
                                                            uint64_t salt, uint32_t *sink)
{
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t acc = 0;
    for (uint64_t i = 0; i < per_thread; i++) {
        uint64_t h = mix64(salt + tid * per_thread + i);
        uint64_t blk = (uint64_t)(((unsigned __int128)h * n_blocks) >> 64);
        const uint32_t *p = buf + blk * WORDS;
        uint32_t a0, a1, a2, a3, a4, a5, a6, a7;
        asm volatile("ld.global.nc.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3), "=r"(a4), "=r"(a5), "=r"(a6), "=r"(a7)
                     : "l"(p));
        acc ^= a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
        if (WORDS == 16) {
            asm volatile("ld.global.nc.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3), "=r"(a4), "=r"(a5), "=r"(a6), "=r"(a7)
                         : "l"(p + 8));
            acc ^= a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
        }
    }
    if (acc == 0x9e3779b9u) sink[0] = acc;   /* keeps the loads alive */
}

/* one 32-byte load in form MODE (the PTX cache operators and L1/L2 hints) */
#define GS_LD8(OP, p, a)                                                                          \
    asm volatile(OP " {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"                                           \
                 : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3]), "=r"(a[4]), "=r"(a[5]),        \
                   "=r"(a[6]), "=r"(a[7])                                                         \
                 : "l"(p))

template <int MODE>
static __device__ __forceinline__ void gs_ld_mode(const uint32_t *p, uint32_t *a)
{
    if (MODE == 0) GS_LD8("ld.global.nc.v8.u32", p, a);
    else if (MODE == 1) GS_LD8("ld.global.nc.L1::no_allocate.v8.u32", p, a);
    else if (MODE == 2) GS_LD8("ld.global.cg.v8.u32", p, a);
    else if (MODE == 3) GS_LD8("ld.global.cs.v8.u32", p, a);
    else if (MODE == 4) GS_LD8("ld.global.lu.v8.u32", p, a);
    else if (MODE == 5) GS_LD8("ld.global.v8.u32", p, a);
    else if (MODE == 6) GS_LD8("ld.global.cv.v8.u32", p, a);
    else if (MODE == 7) GS_LD8("ld.global.L1::no_allocate.v8.u32", p, a);
    else if (MODE == 8) GS_LD8("ld.global.nc.L1::evict_first.v8.u32", p, a);
    else GS_LD8("ld.global.nc.L2::64B.v8.u32", p, a);
}

template <int MODE>
static __global__ void __launch_bounds__(256) gather_mode_kernel(const uint32_t *__restrict__ buf,
                                                                 uint64_t n_blocks,
                                                                 uint64_t per_thread, uint64_t salt,
                                                                 uint32_t *sink)
{
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t acc = 0;
    for (uint64_t i = 0; i < per_thread; i++) {
        uint64_t h = mix64(salt + tid * per_thread + i);
        uint64_t blk = (uint64_t)(((unsigned __int128)h * n_blocks) >> 64);
        uint32_t a[8];
        gs_ld_mode<MODE>(buf + blk * 8, a);
        acc ^= a[0] ^ a[1] ^ a[2] ^ a[3] ^ a[4] ^ a[5] ^ a[6] ^ a[7];
    }
    if (acc == 0x9e3779b9u) sink[0] = acc;
}

typedef void (*gs_gather_fn)(const uint32_t *, uint64_t, uint64_t, uint64_t, uint32_t *);

extern "C" int gs_probe_random_gather_mode(int device, uint64_t bytes, uint32_t mode,
                                           uint64_t n_loads, double *gbps)
{
    static const gs_gather_fn fns[10] = {
        gather_mode_kernel<0>, gather_mode_kernel<1>, gather_mode_kernel<2>, gather_mode_kernel<3>,
        gather_mode_kernel<4>, gather_mode_kernel<5>, gather_mode_kernel<6>, gather_mode_kernel<7>,
        gather_mode_kernel<8>, gather_mode_kernel<9>};
    if (!gbps || mode > 9 || bytes < 1024 || n_loads == 0) {
        gs_set_error("gs_probe_random_gather_mode: mode 0-9, bytes >= 1024, n_loads > 0");
        return GS_EINVAL;
    }
    GS_ON_DEVICE(device);
    int sms = 0;
    GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    uint32_t *buf = NULL, *sink = NULL;
    GS_CUDA(cudaMalloc(&buf, bytes));
    cudaError_t e = cudaMalloc(&sink, 4);
    cudaEvent_t a = NULL, b = NULL;
    if (e == cudaSuccess) e = cudaMemset(buf, 1, bytes);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    uint64_t n_blocks = bytes / 32;
    uint32_t grid = (uint32_t)sms * 8;
    uint64_t threads = (uint64_t)grid * 256;
    uint64_t per = (n_loads + threads - 1) / threads;
    float best = 1e30f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
        cudaEventRecord(a);
        fns[mode]<<<grid, 256>>>(buf, n_blocks, per, 0x1234 + rep * 77, sink);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return gs_cuda_fail(e, "random gather probe");
    *gbps = (double)(per * threads) * 32 / (best * 1e-3) / 1e9;
    return GS_OK;
}

extern "C" int gs_probe_random_gather(int device, uint64_t bytes, uint32_t load_bytes,
                                      uint64_t n_loads, double *gbps)
{
    if (!gbps || (load_bytes != 32 && load_bytes != 64) || bytes < 1024 || n_loads == 0) {
        gs_set_error("gs_probe_random_gather: load_bytes 32|64, bytes >= 1024, n_loads > 0");
        return GS_EINVAL;
    }
    GS_ON_DEVICE(device);
    int sms = 0;
    GS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    uint32_t *buf = NULL, *sink = NULL;
    GS_CUDA(cudaMalloc(&buf, bytes));
    cudaError_t e = cudaMalloc(&sink, 4);
    cudaEvent_t a = NULL, b = NULL;
    if (e == cudaSuccess) e = cudaMemset(buf, 1, bytes);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    uint64_t n_blocks = bytes / load_bytes;
    uint32_t grid = (uint32_t)sms * 8;
    uint64_t threads = (uint64_t)grid * 256;
    uint64_t per = (n_loads + threads - 1) / threads;
    float best = 1e30f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
        cudaEventRecord(a);
        if (load_bytes == 32) gather_kernel<8><<<grid, 256>>>(buf, n_blocks, per, 0x1234 + rep * 77, sink);
        else gather_kernel<16><<<grid, 256>>>(buf, n_blocks, per, 0x1234 + rep * 77, sink);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms;   /* first launch is warm-up */
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return gs_cuda_fail(e, "random gather probe");
    *gbps = (double)(per * threads) * load_bytes / (best * 1e-3) / 1e9;
    return GS_OK;
}

extern "C" int gs_set_l2_fetch_granularity(int device, int bytes)
{
    if (bytes != 0 && bytes != 32 && bytes != 64 && bytes != 128) {
        gs_set_error("L2 fetch granularity must be 32, 64 or 128 bytes");
        return GS_EINVAL;
    }
    GS_ON_DEVICE(device);
    if (bytes) GS_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)bytes));
    size_t v = 0;
    GS_CUDA(cudaDeviceGetLimit(&v, cudaLimitMaxL2FetchGranularity));
    return (int)v;
}
