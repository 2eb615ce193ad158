// stats.cuh — pieces of the deterministic chunk statistics shared by the
// reduction kernels: a chunk's (n, mean, M2) and the block-wide sum whose
// summation order every reduction kernel follows.
#pragma once
#include <cstdint>

#include "../../include/kontract_gpu.h"

namespace kx {

// Values per chunk: a chunk's statistics do not depend on how many chunks
// or blocks a launch has, so every launch shape gives the same result.
static_assert(KX_STATS_CHUNK == 16384u, "chunk size of the C ABI");

struct ChunkDesc {
    uint64_t begin;
    uint32_t count;
    uint32_t pad;
};
struct ChunkOut {
    double n, mean, m2;
};

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    if (threadIdx.x == 0) red[0] = t;
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

}  // namespace kx
