// paths_gbm.cu — GBM instantiations of the fused path kernel (one scenario).
#include "paths_kernel.cuh"

namespace kx {
template __global__ void k_paths<float, M_GBM, 1, 4>(const PathArgs);
template __global__ void k_paths<float, M_GBM, 1, 3>(const PathArgs);
template __global__ void k_paths<float, M_GBM, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_GBM, 1, 4>(const PathArgs);
template __global__ void k_paths<double, M_GBM, 1, 2>(const PathArgs);

const void *paths_kernel_gbm(int fp64, int minb) {
    if (fp64) return minb >= 4 ? (const void *)&k_paths<double, M_GBM, 1, 4> : (const void *)&k_paths<double, M_GBM, 1, 2>;
    switch (minb) {
    case 4: return (const void *)&k_paths<float, M_GBM, 1, 4>;
    case 3: return (const void *)&k_paths<float, M_GBM, 1, 3>;
    default: return (const void *)&k_paths<float, M_GBM, 1, 2>;
    }
}
}  // namespace kx
