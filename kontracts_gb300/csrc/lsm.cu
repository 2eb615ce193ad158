// lsm.cu — Longstaff-Schwartz American pricing (placeholder until the kernels land).
#include "engine.hpp"
using namespace kx;
extern "C" kx_status kx_price_american_lsm(const kx_program *, const kx_model *, const kx_mc_config *,
                                           const double *, size_t, int32_t, kx_price_result *) {
    return guarded([&] { raise(KX_UNSUPPORTED, "LSM not built yet"); });
}
