// stats.cuh — the deterministic chunk statistics shared by the reduction
// kernels: a chunk's (n, mean, M2) from exact integer sums (device, by a
// cluster of blocks, and its host mirror), and the FP64 passes kept for
// chunks with non-finite values.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstring>

#include "../../include/kontract_gpu.h"
#if defined(__CUDACC__)
#include <cooperative_groups.h>
#endif

namespace kx {

// Values per chunk: a chunk's statistics do not depend on how many chunks
// or blocks a launch has, so every launch shape gives the same result.
static_assert(KX_STATS_CHUNK == 16384u, "chunk size of the C ABI");

// The exact reduction of a chunk of prices: a cluster of KX_STATS_CLUSTER
// blocks of KX_STATS_THREADS threads, 16 values a thread.
#define KX_STATS_CLUSTER 4
#define KX_STATS_THREADS 256

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

// The two FP64 passes over one chunk, by one block: its mean, then the sum of
// squared deviations from it (pricer.rs:303-328 also takes two passes); four
// accumulators a thread (values i, i + B, i + 2B, i + 3B of its stride, B the
// block size), the order of every sum fixed. Used for chunks holding an
// infinity or a NaN, where the integer sums below do not apply.
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

// ---------------------------------------------------------------------------
// Exact chunk statistics in integers. GB300 runs FP64 at about 1/64 of its
// FP32 rate, so the FP64 passes above cost about two SM cycles per value and
// bound the reduction. Here each value becomes a signed integer X, a multiple
// of one unit 2^(E - 1075 - FX_GUARD) where E is the largest exponent field
// in the chunk: X = m << FX_GUARD >> (E - e) for the 53-bit mantissa m and
// exponent field e of the value (truncated toward zero when e < E - FX_GUARD,
// i.e. an error below 2^-54 of the chunk's largest value; exact otherwise).
// Deviations d = X - C from the chunk's first value C are summed exactly,
// S = sum d in 128 bits and Q = sum d^2 in unsigned 128 bits (|X| < 2^55, so
// |d| < 2^56, and at most 2^14 values: neither overflows), and one thread
// turns them into the mean C + S/n and M2 = Q - S^2/n, each rounded once or
// twice. Integer sums do not depend on their order, so the result depends
// only on the chunk's values, on any launch shape, and the host mirror below
// gives the same bits. About 25 integer instructions per value (the squares'
// products as multiply-adds on the FMA pipe, the rest on the ALU pipe)
// replace 3 FP64 ones. Chunks holding an infinity or a NaN take the FP64
// passes.
// ---------------------------------------------------------------------------
#if defined(__CUDACC__)
#define KX_HD __host__ __device__
#else
#define KX_HD
#endif
constexpr int FX_GUARD = 2;  // fraction bits kept below the largest value's last mantissa bit
typedef __int128 fx_i128;
typedef unsigned __int128 fx_u128;

KX_HD inline uint64_t fx_bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}
KX_HD inline uint32_t fx_expo(double x) { return (uint32_t)(fx_bits(x) >> 52) & 0x7FFu; }

// x in units of 2^(E - 1075 - FX_GUARD), E >= 1 and >= the exponent field of x.
KX_HD inline int64_t fx_value(double x, uint32_t E) {
    const uint64_t b = fx_bits(x);
    const uint32_t ef = (uint32_t)(b >> 52) & 0x7FFu;
    uint64_t m = b & 0x000FFFFFFFFFFFFFull;
    if (ef) m |= 0x0010000000000000ull;  // the implicit bit (subnormals have none and e = 1)
    const uint32_t t = E - (ef ? ef : 1u);
#if defined(__CUDA_ARCH__)
    asm("shr.b64 %0, %1, %2;" : "=l"(m) : "l"(m << FX_GUARD), "r"(t));  // PTX: a shift of 64 or more gives 0
#else
    m = t < 64u ? (m << FX_GUARD) >> t : 0ull;
#endif
    const int64_t s = (int64_t)b >> 63;  // 0 or -1: the sign
    return ((int64_t)m ^ s) - s;
}

// d^2 for |d| < 2^57 from three 32 x 32 -> 64 products.
KX_HD inline fx_u128 fx_square(int64_t d) {
    const uint64_t a = d < 0 ? 0ull - (uint64_t)d : (uint64_t)d;
    const uint32_t lo = (uint32_t)a, hi = (uint32_t)(a >> 32);
    const uint64_t ll = (uint64_t)lo * lo, lh = (uint64_t)lo * hi, hh = (uint64_t)hi * hi;
    return ((fx_u128)hh << 64) + ((fx_u128)(lh << 1) << 32) + ll;
}

KX_HD inline double fx_u128_to_double(fx_u128 v) {  // round-to-nearest of each half; hi * 2^64 is exact
    return (double)(uint64_t)(v >> 64) * 18446744073709551616.0 + (double)(uint64_t)v;
}
KX_HD inline double fx_i128_to_double(fx_i128 v) {
    return (double)(int64_t)(v >> 64) * 18446744073709551616.0 + (double)(uint64_t)v;
}

// 2^k for -1022 <= k <= 1023, from its bits.
KX_HD inline double fx_pow2(int k) {
    const uint64_t b = (uint64_t)(k + 1023) << 52;
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}

// x * 2^k by exact power-of-two steps (one rounding at most, where the result
// is subnormal).
KX_HD inline double fx_scale(double x, int k) {
    while (k > 1000) {
        x *= 0x1p1000;
        k -= 1000;
    }
    while (k < -1000) {
        x *= 0x1p-1000;
        k += 1000;
    }
    return x * fx_pow2(k);
}

// The chunk's mean and M2 from the exact sums (n values, first value C).
KX_HD inline void fx_finish(int64_t C, fx_i128 S, fx_u128 Q, uint32_t n, uint32_t E, double &mean, double &m2) {
    // S = q n + r with |r| < n: q from a rounded quotient, then corrected exactly
    const int64_t q1 = (int64_t)(fx_i128_to_double(S) / (double)n);
    const int64_t r1 = (int64_t)(S - (fx_i128)q1 * (fx_i128)n);
    const int64_t q2 = r1 / (int64_t)n;
    const int64_t q = q1 + q2, r = r1 - q2 * (int64_t)n;
    // n M2 = n Q - S^2, so M2 = (Q - q^2 n - 2 q r) - r^2 / n; the bracket is an
    // integer in [0, 2^128), exact in wrapping unsigned arithmetic
    const fx_u128 T = Q - fx_square(q) * (fx_u128)n - (fx_u128)((fx_i128)(2 * q) * (fx_i128)r);
    const double m2u = fx_u128_to_double(T) - (double)(r * r) / (double)n;
    const double mu = (double)(C + q) + (double)r / (double)n;
    const int k = (int)E - 1075 - FX_GUARD;
    mean = fx_scale(mu, k);
    m2 = fx_scale(m2u, 2 * k);
}

// Sums of S (signed) and Q (unsigned) over a warp, 128 bits each.
__device__ __forceinline__ void fx_warp_sum(fx_i128 &S, fx_u128 &Q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t slo = __shfl_xor_sync(0xffffffffu, (unsigned long long)(uint64_t)S, o);
        const uint64_t shi = __shfl_xor_sync(0xffffffffu, (unsigned long long)(uint64_t)(S >> 64), o);
        const uint64_t qlo = __shfl_xor_sync(0xffffffffu, (unsigned long long)(uint64_t)Q, o);
        const uint64_t qhi = __shfl_xor_sync(0xffffffffu, (unsigned long long)(uint64_t)(Q >> 64), o);
        S += (fx_i128)(((fx_u128)shi << 64) | slo);
        Q += ((fx_u128)qhi << 64) | qlo;
    }
}

// Cluster barrier phases (PTX barrier.cluster): every thread of every block
// of the cluster arrives, then waits for all of them. `release` / `acquire`
// order the distributed shared memory writes before the barrier with the
// reads after it.
__device__ __forceinline__ void cluster_arrive_relaxed() { asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_arrive_release() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait_acquire() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// The exact statistics of one chunk of values val(i), 1 <= count <=
// KX_STATS_CHUNK (a price, or an estimator formed per path in FP64 from
// weighted scenarios), by a cluster of CS blocks of NT threads:
// block r of the cluster holds values r * NT * VPT .. (r + 1) * NT * VPT - 1
// of the chunk in registers, VPT a thread, all loaded at once. A block of NT
// threads at 64 registers leaves room for 65536 / (64 NT) resident blocks a
// multiprocessor, so one block's loads overlap another's integer work. The
// blocks push their exponent maxima into every block's shared memory and
// their sums into block 0's (distributed shared memory), so every read is
// local and the other blocks leave while block 0 forms the result. Every
// block passes the same three barrier phases: (A) all blocks have started
// (arrived before the loads complete, waited on before the first remote
// write), (B) every maximum is written, (C) every sum is written. Smem:
// `emax` NW + CS words, `part` 4 (NW + CS) words, `red` 32 doubles (FP64
// passes of a non-finite chunk, run by block 0). mean and m2 are valid in
// thread 0 of block 0 of the cluster.
template <int CS, int NT, class Val>
__device__ __forceinline__ void chunk_moments_exact_cluster(const Val &val, uint32_t count, uint32_t *emax,
                                                            uint64_t *part, double *red, double &mean, double &m2) {
    constexpr int NW = NT / 32, VPT = (int)KX_STATS_CHUNK / (CS * NT);
    static_assert(VPT * CS * NT == (int)KX_STATS_CHUNK && NT % 32 == 0, "cluster shape");
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t rank = cl.block_rank(), base = rank * (uint32_t)(NT * VPT);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    double x[VPT];
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
        const uint32_t i = base + threadIdx.x + (uint32_t)(k * NT);
        x[k] = i < count ? val(i) : 0.0;  // past the end: exponent field 0, excluded from the sums below
    }
    cluster_arrive_relaxed();  // (A) this block has started
    uint32_t e = 0;
#pragma unroll
    for (int k = 0; k < VPT; ++k) e = max(e, fx_expo(x[k]));
    e = __reduce_max_sync(0xffffffffu, e);
    if (l == 0) emax[w] = e;
    __syncthreads();
    cluster_wait_acquire();  // (A) every block has started: remote writes are safe
    if (w == 0) {
        const uint32_t t = __reduce_max_sync(0xffffffffu, l < NW ? emax[l] : 0u);
        if (l < CS) *cl.map_shared_rank(emax + NW + rank, l) = t;  // this block's maximum, to block l
    }
    cluster_arrive_release();
    cluster_wait_acquire();  // (B) every maximum is in every block
    uint32_t E = 0;
#pragma unroll
    for (int r = 0; r < CS; ++r) E = max(E, emax[NW + r]);
    if (E == 0x7FFu) {  // an infinity or a NaN: block 0 runs the FP64 passes over the chunk
        if (rank == 0) chunk_moments(val, count, red, mean, m2);
        cluster_arrive_relaxed();
        cluster_wait_acquire();  // (C)
        return;
    }
    if (E == 0u) E = 1u;
    const int64_t C = fx_value(val(0), E);  // value 0 of the chunk
    // d = dh 2^29 + dl (0 <= dl < 2^29, |dh| < 2^27 as |d| < 2^56): d^2 = dl^2 +
    // 2^30 dl dh + 2^58 dh^2, each product a 32 x 32 -> 64 multiply-add into a
    // 64-bit sum that VPT <= 16 values cannot overflow (< 2^62)
    static_assert(VPT <= 16, "64-bit partial sums of the squares");
    int64_t S1 = 0;  // |S1| < VPT * 2^56
    uint64_t qll = 0;
    int64_t qlh = 0, qhh = 0;
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
        if (base + threadIdx.x + (uint32_t)(k * NT) < count) {
            const int64_t d = fx_value(x[k], E) - C;
            S1 += d;
            const uint32_t dl = (uint32_t)d & 0x1FFFFFFFu;
            const int32_t dh = (int32_t)(d >> 29);
            qll += (uint64_t)dl * dl;
            qlh += (int64_t)dh * (int32_t)dl;
            qhh += (int64_t)dh * dh;
        }
    }
    fx_u128 Q = (fx_u128)((fx_i128)qll + ((fx_i128)qlh << 30) + ((fx_i128)qhh << 58));
    fx_i128 S = S1;
    fx_warp_sum(S, Q);
    if (l == 0) {
        part[4 * w] = (uint64_t)S;
        part[4 * w + 1] = (uint64_t)(S >> 64);
        part[4 * w + 2] = (uint64_t)Q;
        part[4 * w + 3] = (uint64_t)(Q >> 64);
    }
    __syncthreads();
    if (w == 0) {
        S = 0;
        Q = 0;
        if (l < NW) {
            S = (fx_i128)(((fx_u128)part[4 * l + 1] << 64) | part[4 * l]);
            Q = ((fx_u128)part[4 * l + 3] << 64) | part[4 * l + 2];
        }
        fx_warp_sum(S, Q);
        if (l < 4) {  // this block's sums, to block 0
            const uint64_t word = l == 0 ? (uint64_t)S : l == 1 ? (uint64_t)(S >> 64) : l == 2 ? (uint64_t)Q
                                                                                                  : (uint64_t)(Q >> 64);
            *cl.map_shared_rank(part + 4 * NW + 4 * rank + l, 0) = word;
        }
    }
    cluster_arrive_release();
    cluster_wait_acquire();  // (C) every block's sums are in block 0
    if (rank == 0 && threadIdx.x == 0) {
        fx_i128 St = 0;
        fx_u128 Qt = 0;
        for (int r = 0; r < CS; ++r) {
            const uint64_t *p = part + 4 * NW + 4 * r;
            St += (fx_i128)(((fx_u128)p[1] << 64) | p[0]);
            Qt += ((fx_u128)p[3] << 64) | p[2];
        }
        fx_finish(C, St, Qt, count, E, mean, m2);
    }
}

// Host mirror of chunk_moments_exact_cluster: the same bits for finite
// values a[i], or a[i] - b[i] rounded to FP64 (as the device forms the
// estimator of weights {1, -1}). A chunk with an infinity or a NaN gets the
// plain two-pass FP64 result, of the same IEEE class as the device's.
inline void chunk_moments_exact_host(const double *a, const double *b, uint32_t count, double &mean, double &m2) {
    mean = m2 = 0.0;
    if (count == 0) return;
    auto val = [&](uint32_t i) { return b ? a[i] - b[i] : a[i]; };
    uint32_t E = 0;
    for (uint32_t i = 0; i < count; ++i) E = std::max(E, fx_expo(val(i)));
    if (E == 0x7FFu) {
        double s = 0.0;
        for (uint32_t i = 0; i < count; ++i) s += val(i);
        mean = s / (double)count;
        for (uint32_t i = 0; i < count; ++i) m2 += (val(i) - mean) * (val(i) - mean);
        return;
    }
    if (E == 0u) E = 1u;
    const int64_t C = fx_value(val(0), E);
    fx_i128 S = 0;
    fx_u128 Q = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const int64_t d = fx_value(val(i), E) - C;
        S += d;
        Q += fx_square(d);
    }
    fx_finish(C, S, Q, count, E, mean, m2);
}

}  // namespace kx
