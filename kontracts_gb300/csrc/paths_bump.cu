// paths_bump.cu — GBM instantiations with seven bump scenarios sharing each
// path's normals (greeks.rs:60-98 reprices in one launch).
#include "paths_kernel.cuh"

namespace kx {
template __global__ void k_paths<float, M_GBM, KX_MAX_NS, 2>(const PathArgs);
template __global__ void k_paths<float, M_GBM, KX_MAX_NS, 1>(const PathArgs);
template __global__ void k_paths<double, M_GBM, KX_MAX_NS, 1>(const PathArgs);

const void *paths_kernel_bump(int fp64, int minb) {
    if (fp64) return (const void *)&k_paths<double, M_GBM, KX_MAX_NS, 1>;
    return minb >= 2 ? (const void *)&k_paths<float, M_GBM, KX_MAX_NS, 2> : (const void *)&k_paths<float, M_GBM, KX_MAX_NS, 1>;
}
}  // namespace kx
