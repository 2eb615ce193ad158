// capi.cpp — host-only entry points of the C ABI (include/kontract_gpu.h):
// compilation of contracts, plan and grid queries, error reporting.
#include <cstring>
#include <new>

#include "capi_util.hpp"
#include "frontend.hpp"

struct kx_program {
    kx::Program p;
};

namespace kx {
thread_local std::string g_last_error;
thread_local double g_last_error_time = __builtin_nan("");
thread_local uint64_t g_last_error_step = UINT64_MAX;

kx_status fail_status(const Error &e) {
    g_last_error = e.msg;
    g_last_error_time = e.time;
    g_last_error_step = e.step;
    return e.code;
}
const Program &program_of(const kx_program *h, bool need_lowered) {
    if (!h) raise(KX_INVALID_ARGUMENT, "program handle is NULL");
    h->p.check(need_lowered);
    return h->p;
}
}  // namespace kx

using namespace kx;

extern "C" {

int32_t kx_abi_version(void) { return KX_ABI_VERSION; }

const char *kx_last_error_message(void) { return g_last_error.c_str(); }

kx_status kx_last_error_payload(double *time, uint64_t *step) {
    if (time) *time = g_last_error_time;
    if (step) *step = g_last_error_step;
    return KX_OK;
}

kx_status kx_compile(const char *contract_json, kx_program **out) {
    return guarded([&] {
        if (!out) raise(KX_INVALID_ARGUMENT, "out is NULL");
        *out = nullptr;
        auto *h = new (std::nothrow) kx_program();
        if (!h) raise(KX_INVALID_ARGUMENT, "out of host memory");
        try {
            h->p.json = contract_json ? contract_json : "";
            h->p.ast = parse_contract_json(contract_json);
            try {
                h->p.plan = compile_plan(*h->p.ast);
                try {
                    lower(h->p);
                } catch (const Error &e) {
                    h->p.low_status = e.code;
                    h->p.low_msg = e.msg;
                }
            } catch (const Error &e) {
                h->p.plan_status = e.code;
                h->p.plan_msg = e.msg;
            }
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

void kx_program_free(kx_program *prog) { delete prog; }

kx_status kx_program_plan(const kx_program *prog, kx_plan_info *info, double *fixed_dates, size_t dates_cap,
                          char *assets_buf, size_t assets_cap) {
    return guarded([&] {
        const Program &p = program_of(prog, false);
        if (!info) raise(KX_INVALID_ARGUMENT, "info is NULL");
        info->n_assets = (uint32_t)p.plan.assets.size();
        info->n_fixed_dates = (uint32_t)p.plan.fixed_dates.size();
        info->horizon = p.plan.horizon;
        info->needs_fine_grid = p.plan.needs_fine_grid ? 1 : 0;
        info->n_triggers = p.low.prog.n_trig;
        info->n_flows = p.low.prog.n_leaf;
        info->n_accumulators = p.low.prog.n_acc;
        if (fixed_dates)
            for (size_t i = 0; i < p.plan.fixed_dates.size() && i < dates_cap; ++i) fixed_dates[i] = p.plan.fixed_dates[i];
        if (assets_buf && assets_cap) {
            std::string s;
            for (size_t i = 0; i < p.plan.assets.size(); ++i) {
                if (i) s += '\n';
                s += p.plan.assets[i];
            }
            strncpy(assets_buf, s.c_str(), assets_cap - 1);
            assets_buf[assets_cap - 1] = 0;
        }
    });
}

kx_status kx_time_grid(const kx_program *prog, uint32_t steps_per_year, int32_t force_fine, double *out, size_t cap,
                       size_t *n) {
    return guarded([&] {
        const Program &p = program_of(prog, false);
        if (!n) raise(KX_INVALID_ARGUMENT, "n is NULL");
        auto g = time_grid_forced(p.plan, steps_per_year, force_fine != 0);
        *n = g.size();
        if (out)
            for (size_t i = 0; i < g.size() && i < cap; ++i) out[i] = g[i];
    });
}

}  // extern "C"
