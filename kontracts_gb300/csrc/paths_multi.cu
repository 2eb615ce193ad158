// paths_multi.cu — the path kernel of correlated multi-factor GBM
// (CorrelatedGbmN, multi_asset.rs:107-170): baskets, spreads and any other
// contract on several spots, through the general event handler.
#include "paths_kernel.cuh"

namespace kx {
template __global__ void k_paths<float, M_MULTI, 1, 4>(const PathArgs);
template __global__ void k_paths<float, M_MULTI, 1, 3>(const PathArgs);
template __global__ void k_paths<float, M_MULTI, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_MULTI, 1, 2>(const PathArgs);

const void *paths_kernel_multi(int fp64, int minb) {
    if (fp64) return (const void *)&k_paths<double, M_MULTI, 1, 2>;
    switch (minb) {
    case 4: return (const void *)&k_paths<float, M_MULTI, 1, 4>;
    case 3: return (const void *)&k_paths<float, M_MULTI, 1, 3>;
    default: return (const void *)&k_paths<float, M_MULTI, 1, 2>;
    }
}
}  // namespace kx
