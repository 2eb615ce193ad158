// paths_heston.cu — Heston instantiations of the fused path kernels.
#include "paths_lean.cuh"

namespace kx {
template __global__ void k_paths<float, M_HESTON, 1, 4>(const PathArgs);
template __global__ void k_paths<float, M_HESTON, 1, 3>(const PathArgs);
template __global__ void k_paths<float, M_HESTON, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_HESTON, 1, 2>(const PathArgs);
template __global__ void k_lean<float, M_HESTON, 6>(const PathArgs);
template __global__ void k_lean<float, M_HESTON, 5>(const PathArgs);
template __global__ void k_lean<float, M_HESTON, 4>(const PathArgs);
template __global__ void k_lean<double, M_HESTON, 3>(const PathArgs);

const void *paths_kernel_heston(int fp64, int minb) {
    if (fp64) return (const void *)&k_paths<double, M_HESTON, 1, 2>;
    switch (minb) {
    case 4: return (const void *)&k_paths<float, M_HESTON, 1, 4>;
    case 3: return (const void *)&k_paths<float, M_HESTON, 1, 3>;
    default: return (const void *)&k_paths<float, M_HESTON, 1, 2>;
    }
}

const void *lean_kernel_heston(int fp64, int minb) {
    if (fp64) return (const void *)&k_lean<double, M_HESTON, 3>;
    switch (minb) {
    case 6: return (const void *)&k_lean<float, M_HESTON, 6>;
    case 5: return (const void *)&k_lean<float, M_HESTON, 5>;
    default: return (const void *)&k_lean<float, M_HESTON, 4>;
    }
}
}  // namespace kx
