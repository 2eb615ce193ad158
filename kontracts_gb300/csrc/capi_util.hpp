// capi_util.hpp — exception-to-status plumbing shared by the C ABI sources.
#pragma once
#include <cstdint>
#include <exception>
#include <string>

#include "frontend.hpp"

struct kx_program;

namespace kx {
extern thread_local std::string g_last_error;
extern thread_local double g_last_error_time;    // payload of KX_TIME_OUT_OF_RANGE, else NaN
extern thread_local uint64_t g_last_error_step;  // payload of KX_STEP_OUT_OF_RANGE, else UINT64_MAX
kx_status fail_status(const Error &e);
const Program &program_of(const kx_program *h, bool need_lowered = true);

// Run `f`, translating exceptions into kx_status and the thread's message.
template <class F>
kx_status guarded(F &&f) {
    try {
        f();
        g_last_error.clear();
        g_last_error_time = __builtin_nan("");
        g_last_error_step = UINT64_MAX;
        return KX_OK;
    } catch (const Error &e) {
        return fail_status(e);
    } catch (const std::bad_alloc &) {
        return fail_status(Error{KX_INVALID_ARGUMENT, "out of host memory"});
    } catch (const std::exception &e) {
        return fail_status(Error{KX_INVALID_ARGUMENT, e.what()});
    }
}
}  // namespace kx
