// paths_pair.cu — the coarse path kernels of multilevel Monte-Carlo pairs: GBM
// and Heston paths whose steps consume the normals of two fine steps
// (simulator.rs:321-409, 592-690).
#include "paths_kernel.cuh"

namespace kx {
template __global__ void k_paths<float, M_GBM_PAIR, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_GBM_PAIR, 1, 2>(const PathArgs);
template __global__ void k_paths<float, M_HESTON_PAIR, 1, 2>(const PathArgs);
template __global__ void k_paths<double, M_HESTON_PAIR, 1, 2>(const PathArgs);

const void *paths_kernel_pair(int model, int fp64) {
    if (model == KX_MODEL_GBM)
        return fp64 ? (const void *)&k_paths<double, M_GBM_PAIR, 1, 2> : (const void *)&k_paths<float, M_GBM_PAIR, 1, 2>;
    return fp64 ? (const void *)&k_paths<double, M_HESTON_PAIR, 1, 2> : (const void *)&k_paths<float, M_HESTON_PAIR, 1, 2>;
}
}  // namespace kx
