// paths_pair.cu — the coarse path kernels of multilevel Monte-Carlo pairs: GBM
// and Heston paths whose steps consume the normals of two fine steps
// (simulator.rs:321-409, 592-690). k_lean serves the contracts it serves for
// plain paths (barriers, time events, one running average); k_paths the rest.
#include "paths_lean.cuh"

namespace kx {
template __global__ void k_paths<float, M_GBM_PAIR, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_GBM_PAIR, 1, 2>(const PathArgs);
template __global__ void k_paths<float, M_HESTON_PAIR, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_HESTON_PAIR, 1, 2>(const PathArgs);

#define KX_LEAN_PAIR(R, M, B)                                        \
    template __global__ void k_lean<R, M, B, false>(const PathArgs); \
    template __global__ void k_lean<R, M, B, true>(const PathArgs);  \
    template __global__ void k_lean<R, M, B, true, true>(const PathArgs);
KX_LEAN_PAIR(float, M_GBM_PAIR, 4)
KX_LEAN_PAIR(double, M_GBM_PAIR, 4)
KX_LEAN_PAIR(float, M_HESTON_PAIR, 4)
KX_LEAN_PAIR(double, M_HESTON_PAIR, 3)
#undef KX_LEAN_PAIR

const void *paths_kernel_pair(int model, int fp64) {
    if (model == KX_MODEL_GBM)
        return fp64 ? (const void *)&k_paths<double, M_GBM_PAIR, 1, 2> : (const void *)&k_paths<float, M_GBM_PAIR, 1, 2>;
    return fp64 ? (const void *)&k_paths<double, M_HESTON_PAIR, 1, 2> : (const void *)&k_paths<float, M_HESTON_PAIR, 1, 2>;
}

template <class Real, int M, int B>
static const void *lean_pair_pick(bool stat, bool acc) {
    if (acc) return (const void *)&k_lean<Real, M, B, true, true>;
    return stat ? (const void *)&k_lean<Real, M, B, true> : (const void *)&k_lean<Real, M, B, false>;
}

const void *lean_kernel_pair(int model, int fp64, bool stat, bool acc) {
    if (model == KX_MODEL_GBM)
        return fp64 ? lean_pair_pick<double, M_GBM_PAIR, 4>(stat, acc) : lean_pair_pick<float, M_GBM_PAIR, 4>(stat, acc);
    return fp64 ? lean_pair_pick<double, M_HESTON_PAIR, 3>(stat, acc)
                : lean_pair_pick<float, M_HESTON_PAIR, 4>(stat, acc);
}
}  // namespace kx
