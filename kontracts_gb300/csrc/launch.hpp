// launch.hpp — host-side pieces of a path-kernel launch, shared by the CUDA
// translation units that launch the path kernels (engine.cu and others).
#pragma once
#include <vector>

#include "engine.hpp"
#include "paths_lean.cuh"

namespace kx {

struct Job {  // one contract of a launch
    KxProgram prog;
    StepTables tab;
    ContractDev dev;
    Model model;
    std::vector<double> thr;  // [KX_MAX_NS][KX_MAX_SPOT] log(B / s0_s)
};

// Scenario parameters (bump scenarios share the normals of a path).
struct Scenario {
    double s0, mu, sigma, rate;
};

// Validates an mc config (Philox or shared draws, FP32 / FP64, n_paths < 2^32).
void check_cfg(const kx_mc_config *cfg);

// Binds a lowered contract to a model, a grid and its scenarios.
Job make_job(const Program &p, const Model &m, const kx_mc_config &cfg, const std::vector<double> &grid,
             const std::vector<Scenario> &scen_in, int smooth, double smooth_w);

// Appends the step table of `t` in the launch precision.
template <class Real>
void pack_steps(const StepTables &t, std::vector<unsigned char> &out);

// Path kernel for a model, precision, scenario count and register budget.
const void *select_kernel(int model, bool f64, int ns, int minb, bool lean);

// Whether the lean kernel serves these jobs (KX_PATH_KERNEL may force the general one).
bool use_lean(const std::vector<Job> &jobs, int ns);

// Register budgets (minimum resident blocks per SM) of a kernel family; the
// first is the default when no tuning result is at hand.
const int *variants(int model, bool f64, int ns, bool lean, int &n);

// Per-call bookkeeping of the launch statistics.
void begin_call(Ctx &c);
void end_call(Ctx &c);

}  // namespace kx
