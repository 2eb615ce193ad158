/* A plain C caller of the engine, compiled with gcc against
 * include/kontract_gpu.h only: what a Rust (or any FFI) binding does through
 * the same symbols. It compiles a contract, prices it, takes its pathwise
 * sensitivities, prices an American put and takes a chunk's statistics on the
 * host, and prints one line per call:
 *   <call> <status> <values...>
 * Without a CUDA device the pricing calls return KX_NO_DEVICE; compilation,
 * plan and grid queries never need one. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "kontract_gpu.h"

static const char *UP_AND_OUT =
    "{\"Until\":[{\"Ge\":[{\"Spot\":\"S\"},{\"Const\":200.0}]},{\"When\":[{\"At\":1.0},{\"Scale\":[{\"Max\":"
    "[{\"Sub\":[{\"Spot\":\"S\"},{\"Const\":100.0}]},{\"Const\":0.0}]},{\"One\":\"USD\"}]}]}]}";
static const char *PUT =
    "{\"Scale\":[{\"Max\":[{\"Sub\":[{\"Const\":40.0},{\"Spot\":\"S\"}]},{\"Const\":0.0}]},{\"One\":\"USD\"}]}";

int main(void) {
    printf("abi_version %d %d\n", KX_OK, kx_abi_version());
    kx_program *uo = NULL, *put = NULL, *bad = NULL;
    kx_status st = kx_compile(UP_AND_OUT, &uo);
    printf("compile %d\n", st);
    if (st != KX_OK) return 1;
    st = kx_compile("{\"Nope\":1}", &bad);
    printf("compile_bad %d %s\n", st, bad == NULL ? "null" : "set");
    kx_plan_info info;
    st = kx_program_plan(uo, &info, NULL, 0, NULL, 0);
    printf("plan %d %u %.17g %d\n", st, info.n_assets, info.horizon, info.needs_fine_grid);
    size_t n_grid = 0;
    st = kx_time_grid(uo, 365, 0, NULL, 0, &n_grid);
    printf("grid %d %zu\n", st, n_grid);

    kx_model gbm;
    memset(&gbm, 0, sizeof gbm);
    gbm.kind = KX_MODEL_GBM;
    gbm.s0 = 180.0;
    gbm.mu = 0.05;
    gbm.sigma = 0.25;
    gbm.asset = "S";
    kx_mc_config cfg = {200000, 42, 365, KX_RNG_PHILOX, KX_PREC_FP32, 0, 0.05};
    kx_price_result res;
    memset(&res, 0, sizeof res);
    st = kx_price(uo, &gbm, &cfg, &res, NULL);
    printf("price %d %.17g %.17g %llu\n", st, res.price, res.std_error, (unsigned long long)res.n_paths);

    kx_adjoint_cfg acfg = {16, 0, 0.0};
    kx_sens sens;
    memset(&sens, 0, sizeof sens);
    st = kx_greeks_adjoint(uo, &gbm, &cfg, &acfg, &sens);
    printf("adjoint %d %.17g %.17g %.17g %.17g %.17g\n", st, sens.price, sens.d_s0, sens.d_sigma, sens.d_r,
           sens.smoothing_width);

    st = kx_compile(PUT, &put);
    printf("compile_put %d\n", st);
    kx_model g40 = gbm;
    g40.s0 = 36.0;
    g40.mu = 0.06;
    g40.sigma = 0.2;
    kx_mc_config lcfg = {100000, 7, 50, KX_RNG_PHILOX, KX_PREC_FP64, 0, 0.06};
    double dates[50];
    for (int i = 0; i < 50; ++i) dates[i] = (i + 1) / 50.0;
    memset(&res, 0, sizeof res);
    st = kx_price_american_lsm(put, &g40, &lcfg, dates, 50, 4, &res);
    printf("lsm %d %.17g %.17g %llu\n", st, res.price, res.std_error, (unsigned long long)res.n_paths);

    /* errors: an unknown asset is KX_UNKNOWN_ASSET with the reference's message */
    kx_model other = gbm;
    other.asset = "T";
    st = kx_price(uo, &other, &cfg, &res, NULL);
    double t = 0.0;
    uint64_t k = 0;
    kx_last_error_payload(&t, &k);
    printf("unknown_asset %d %d %d\n", st, isnan(t) ? 1 : 0, k == UINT64_MAX ? 1 : 0);
    /* statistics of a chunk of values on the host (no device): n, mean, M2 */
    const double vals[4] = {1.0, 2.0, 3.0, 4.0};
    kx_chunk_stats cs;
    memset(&cs, 0, sizeof cs);
    st = kx_chunk_moments(vals, NULL, 4u, &cs);
    printf("chunk_moments %d %.17g %.17g %.17g\n", st, cs.n, cs.mean, cs.m2);

    kx_program_free(uo);
    kx_program_free(put);
    return 0;
}
