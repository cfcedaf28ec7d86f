/*
 * gpuseed_tools.h -- measurement probes of libgpuseed.so.  No counterpart in
 * the reference: they measure the hardware the seeding path runs on.
 */
#ifndef GPUSEED_TOOLS_H
#define GPUSEED_TOOLS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Random-gather roofline: n_loads independent loads of load_bytes (32 or 64)
 * at uniformly random aligned addresses of a device buffer of `bytes` bytes
 * (choose bytes > L2).  *gbps = loaded bytes per second / 1e9, best of three
 * timed launches after one warm-up launch. */
int gs_probe_random_gather(int device, uint64_t bytes, uint32_t load_bytes, uint64_t n_loads,
                           double *gbps);

/* The same with 32-byte loads in one of ten load forms: 0 ld.global.nc,
 * 1 .nc.L1::no_allocate, 2 .cg, 3 .cs, 4 .lu, 5 ld.global, 6 .cv,
 * 7 .L1::no_allocate, 8 .nc.L1::evict_first, 9 .nc.L2::64B. */
int gs_probe_random_gather_mode(int device, uint64_t bytes, uint32_t mode, uint64_t n_loads,
                                double *gbps);

/* Largest L2 fetch from DRAM per miss for this process's context on `device`
 * (cudaLimitMaxL2FetchGranularity: 32, 64 or 128; 0 only reads it).  Returns
 * the value in effect (or a negative GS_E* code).  A context limit: it ends
 * with the process and changes no GPU setting. */
int gs_set_l2_fetch_granularity(int device, int bytes);

#ifdef __cplusplus
}
#endif
#endif
