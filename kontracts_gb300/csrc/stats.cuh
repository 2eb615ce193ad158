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

// The two passes over one chunk: its mean, then the sum of squared deviations
// from it (pricer.rs:303-328 also takes two passes). GB300's FP64 units are
// few and the values are FP64, so the loops spend one FP64 operation per
// value in the first pass and two in the second, and every thread keeps four
// accumulators (values i, i + B, i + 2B, i + 3B of its stride, B the block
// size) so that their adds overlap; the order of every sum is fixed.
template <class Val>
__device__ __forceinline__ void chunk_moments(const Val &val, uint32_t count, double *red, double &mean, double &m2) {
    const uint32_t B = blockDim.x;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    uint32_t i = threadIdx.x;
    for (; i + 3 * B < count; i += 4 * B) {
        a0 += val(i);
        a1 += val(i + B);
        a2 += val(i + 2 * B);
        a3 += val(i + 3 * B);
    }
    for (; i < count; i += B) a0 += val(i);
    mean = block_sum((a0 + a1) + (a2 + a3), red) / (double)count;
    double b0 = 0.0, b1 = 0.0, b2 = 0.0, b3 = 0.0;
    i = threadIdx.x;
    for (; i + 3 * B < count; i += 4 * B) {
        const double d0 = val(i) - mean, d1 = val(i + B) - mean, d2 = val(i + 2 * B) - mean,
                     d3 = val(i + 3 * B) - mean;
        b0 = fma(d0, d0, b0);
        b1 = fma(d1, d1, b1);
        b2 = fma(d2, d2, b2);
        b3 = fma(d3, d3, b3);
    }
    for (; i < count; i += B) {
        const double d = val(i) - mean;
        b0 = fma(d, d, b0);
    }
    m2 = block_sum((b0 + b1) + (b2 + b3), red);
}

}  // namespace kx
