/*
 * shim.h -- lets the reference's CUDA kernel bodies compile as host C++.
 *
 * TEST INFRASTRUCTURE ONLY.  CUDA qualifiers become nothing, the vector
 * types become plain structs, threadIdx/blockIdx/blockDim read the emulated
 * thread that is running (emu.cpp), __shfl_up_sync goes to the warp
 * emulator and atomicAdd is a plain add (one host thread runs a launch).
 */
#ifndef GS_REF_SHIM_H
#define GS_REF_SHIM_H

#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned int uint;
struct uint2 { uint32_t x, y; };
struct int2 { int32_t x, y; };
struct uint4 { uint32_t x, y, z, w; };
static inline uint2 make_uint2(uint32_t a, uint32_t b) { uint2 r = {a, b}; return r; }
static inline int2 make_int2(int32_t a, int32_t b) { int2 r = {a, b}; return r; }

struct EmuDim { unsigned x, y, z; };
struct EmuThread { EmuDim tid, bid, bdim; };
extern thread_local EmuThread *emu_cur;

#define threadIdx (emu_cur->tid)
#define blockIdx (emu_cur->bid)
#define blockDim (emu_cur->bdim)
#define __global__
#define __device__
#define __constant__
#define __popc(x) __builtin_popcount((unsigned)(x))

uint32_t emu_shfl_up(uint32_t mask, uint32_t v, unsigned delta);
#define __shfl_up_sync(m, v, d) emu_shfl_up((m), (uint32_t)(v), (unsigned)(d))

static inline uint32_t atomicAdd(uint32_t *p, uint32_t v)
{
    uint32_t o = *p;
    *p = o + v;
    return o;
}

#endif
