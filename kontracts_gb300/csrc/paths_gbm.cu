// paths_gbm.cu — GBM instantiations of the fused path kernels (one scenario).
#include "paths_lean.cuh"

namespace kx {
template __global__ void k_paths<float, M_GBM, 1, 4>(const PathArgs);
template __global__ void k_paths<float, M_GBM, 1, 3>(const PathArgs);
template __global__ void k_paths<float, M_GBM, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_GBM, 1, 4>(const PathArgs);
template __global__ void k_paths<double, M_GBM, 1, 2>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 6, false>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 6, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 6, true, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 5, false>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 5, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 5, true, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 3, false>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 3, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 3, true, true>(const PathArgs);  // the accumulator family: no spills at 80
template __global__ void k_lean<float, M_GBM, 4, false>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 4, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 4, true, true>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 4, false>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 4, true>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 4, true, true>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 3, false>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 3, true>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 3, true, true>(const PathArgs);
// smoothed barriers (bumps of the smoothed payoff)
template __global__ void k_lean<float, M_GBM, 6, true, false, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 3, true, false, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 5, true, false, true>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 4, true, false, true>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 4, true, false, true>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 3, true, false, true>(const PathArgs);

const void *paths_kernel_gbm(int fp64, int minb) {
    if (fp64) return minb >= 4 ? (const void *)&k_paths<double, M_GBM, 1, 4> : (const void *)&k_paths<double, M_GBM, 1, 2>;
    switch (minb) {
    case 4: return (const void *)&k_paths<float, M_GBM, 1, 4>;
    case 3: return (const void *)&k_paths<float, M_GBM, 1, 3>;
    default: return (const void *)&k_paths<float, M_GBM, 1, 2>;
    }
}

template <class Real, int MINB>
static const void *lean_pick(bool stat, bool acc, bool sm) {
    if (sm) return stat && !acc ? (const void *)&k_lean<Real, M_GBM, MINB, true, false, true> : nullptr;
    if (acc) return (const void *)&k_lean<Real, M_GBM, MINB, true, true>;
    return stat ? (const void *)&k_lean<Real, M_GBM, MINB, true> : (const void *)&k_lean<Real, M_GBM, MINB, false>;
}

const void *lean_kernel_gbm(int fp64, int minb, bool stat, bool acc, bool sm) {
    if (fp64) return minb >= 4 ? lean_pick<double, 4>(stat, acc, sm) : lean_pick<double, 3>(stat, acc, sm);
    switch (minb) {
    case 6: return lean_pick<float, 6>(stat, acc, sm);
    case 5: return lean_pick<float, 5>(stat, acc, sm);
    case 3: return lean_pick<float, 3>(stat, acc, sm);
    default: return lean_pick<float, 4>(stat, acc, sm);
    }
}
}  // namespace kx
