// engine.hpp — host-side device context shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "capi_util.hpp"
#include "frontend.hpp"

namespace kx {

void cuda_check(cudaError_t e, const char *what);
#define KX_CUDA(call) ::kx::cuda_check((call), #call)

// Growable device buffer owned by the context.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    void ensure(size_t bytes);
    template <class T>
    T *as() const { return static_cast<T *>(p); }
};

// Growable page-locked host buffer: copies from and to it are true
// asynchronous DMA (a pageable source costs a staging copy per call).
struct PinnedBuf {
    void *p = nullptr;
    size_t cap = 0;
    void ensure(size_t bytes);
    template <class T>
    T *as() const { return static_cast<T *>(p); }
};

struct DrawStore {  // host normals for KX_RNG_SHARED_DRAWS
    DevBuf z64, z32;
    bool is64 = false;
    uint64_t n_paths = 0, dpp = 0;
    bool set = false;
};

struct Ctx {
    std::atomic<bool> ready{false};  // set once, after every field below is valid
    int device = 0;
    int sm_count = 0;
    int cc_major = 0, cc_minor = 0;
    std::string name;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // scratch owned by the context
    DevBuf progs, steps, disc, thr, cons, items, counters, pv, chunks, chunk_out, misc, vr, lsm_paths, lsm_value,
        grid_tabs, statics, mlmc, plan, stats_in;
    // host staging of a call's uploads and downloads (path plan, statistics)
    PinnedBuf plan_stage, stats_stage;
    DrawStore draws;
    kx_launch_stats last{};
    bool kahan_stats = false;  // this call's plain statistics in compensated FP32 (KX_PREC_FP32_KAHAN)
    std::mutex mu;
};

// Lazily initialised process context; throws KX_NO_DEVICE without a GPU.
// Thread-safe: the first callers race only for a set-up mutex, one of them
// creates the stream and events, the others wait and then see the result.
Ctx &ctx();

// Persistent grid size for a kernel with `block` threads and `smem` bytes.
int persistent_blocks(const void *kernel, int block, size_t smem);

double now_ms();

// Deterministic statistics of per-path values: returns (n, mean, M2)
// merged over fixed chunks of [begin, begin + n) of `values` (device), with
// values[i] = sum_s w[s] * base[s * stride + i] when ns > 1.
struct Stats {
    double n = 0, mean = 0, m2 = 0;
};
struct StatsJob {
    uint64_t begin = 0, n = 0;
    int ns = 1;
    double w[8] = {1, 0, 0, 0, 0, 0, 0, 0};
};
std::vector<Stats> device_stats(Ctx &c, const double *values, uint64_t stride, const std::vector<StatsJob> &jobs);
kx_price_result finish(const Stats &s);

// Path-kernel valuation of several contracts on one grid with one model and
// seed (engine.cu).
std::vector<Stats> batch_paths(Ctx &c, const std::vector<const Program *> &progs, const Model &m,
                               const kx_mc_config &cfg, const std::vector<double> &grid);

// Portfolio prices (hard barriers) with pathwise sensitivities (adjoint.cu).
void portfolio_adjoint(Ctx &c, size_t n, const kx_program *const *progs, const kx_model *models,
                       const kx_mc_config *cfgs, kx_price_result *out, kx_sens *sens);

}  // namespace kx
