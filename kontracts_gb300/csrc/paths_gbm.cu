// paths_gbm.cu — GBM instantiations of the fused path kernels (one scenario).
#include "paths_lean.cuh"

namespace kx {
template __global__ void k_paths<float, M_GBM, 1, 4>(const PathArgs);
template __global__ void k_paths<float, M_GBM, 1, 3>(const PathArgs);
template __global__ void k_paths<float, M_GBM, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_GBM, 1, 4>(const PathArgs);
template __global__ void k_paths<double, M_GBM, 1, 2>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 6>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 5>(const PathArgs);
template __global__ void k_lean<float, M_GBM, 4>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 4>(const PathArgs);
template __global__ void k_lean<double, M_GBM, 3>(const PathArgs);

const void *paths_kernel_gbm(int fp64, int minb) {
    if (fp64) return minb >= 4 ? (const void *)&k_paths<double, M_GBM, 1, 4> : (const void *)&k_paths<double, M_GBM, 1, 2>;
    switch (minb) {
    case 4: return (const void *)&k_paths<float, M_GBM, 1, 4>;
    case 3: return (const void *)&k_paths<float, M_GBM, 1, 3>;
    default: return (const void *)&k_paths<float, M_GBM, 1, 2>;
    }
}

const void *lean_kernel_gbm(int fp64, int minb) {
    if (fp64) return minb >= 4 ? (const void *)&k_lean<double, M_GBM, 4> : (const void *)&k_lean<double, M_GBM, 3>;
    switch (minb) {
    case 6: return (const void *)&k_lean<float, M_GBM, 6>;
    case 5: return (const void *)&k_lean<float, M_GBM, 5>;
    default: return (const void *)&k_lean<float, M_GBM, 4>;
    }
}
}  // namespace kx
