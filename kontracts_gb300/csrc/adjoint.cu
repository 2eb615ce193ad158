// adjoint.cu — pathwise adjoint Greeks (placeholder until the kernels land).
#include "engine.hpp"
using namespace kx;
extern "C" kx_status kx_greeks_adjoint(const kx_program *, const kx_model *, const kx_mc_config *,
                                       const kx_adjoint_cfg *, kx_sens *) {
    return guarded([&] { raise(KX_UNSUPPORTED, "adjoint not built yet"); });
}
