// capi_util.hpp — exception-to-status plumbing shared by the C ABI sources.
#pragma once
#include <exception>
#include <string>

#include "frontend.hpp"

struct kx_program;

namespace kx {
extern thread_local std::string g_last_error;
kx_status fail_status(const Error &e);
const Program &program_of(const kx_program *h, bool need_lowered = true);

// Run `f`, translating exceptions into kx_status and the thread's message.
template <class F>
kx_status guarded(F &&f) {
    try {
        f();
        g_last_error.clear();
        return KX_OK;
    } catch (const Error &e) {
        return fail_status(e);
    } catch (const std::bad_alloc &) {
        g_last_error = "out of host memory";
        return KX_INVALID_ARGUMENT;
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return KX_INVALID_ARGUMENT;
    }
}
}  // namespace kx
