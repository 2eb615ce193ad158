// launch.hpp — host-side pieces of a path-kernel launch, shared by the CUDA
// translation units that launch the path kernels (engine.cu and others).
#pragma once
#include <vector>

#include "engine.hpp"
#include "paths_lean.cuh"
#include "stats.cuh"

namespace kx {

struct Job {  // one contract of a launch
    KxProgram prog;
    StepTables tab;
    ContractDev dev;
    Model model;
    std::vector<double> thr;  // [KX_MAX_NS][KX_MAX_SPOT] log(B / s0_s)
    uint32_t path_base = 0;   // first path index of the stream this launch prices
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
const void *select_kernel(int model, bool f64, int ns, int minb, bool lean, bool stat = false, bool acc = false,
                          bool sm = false);

// Whether the lean kernel serves these jobs (KX_PATH_KERNEL may force the general one).
bool use_lean(const std::vector<Job> &jobs, int ns);
// Whether some job keeps a running average (the lean kernel's ACC variant).
bool lean_has_average(const std::vector<Job> &jobs);
// Whether some job weighs smoothed barriers (the lean kernel's SM variant).
bool lean_smoothed(const std::vector<Job> &jobs);

// Compiles the static schedule of a job; false when it has none.
bool build_static(const Job &j, StaticDev &T);
// Whether every job of a lean launch has a static schedule (KX_PATH_KERNEL =
// "lean" forces the general event handler of k_lean).
bool use_static(const std::vector<Job> &jobs, int ns);

// Register budgets (minimum resident blocks per SM) of a kernel family; the
// first is the default when no tuning result is at hand.
const int *variants(int model, bool f64, int ns, bool lean, int &n);

// Host-side tables and geometry of one path-kernel launch over `jobs`.
struct PathPlan {
    bool f64 = false, lean = false, stat = false, acc = false, sm = false;
    int model = 0, ns = 1, minb = 0;
    std::vector<KxProgram> progs;
    std::vector<unsigned char> steps, thr;
    std::vector<double> disc;
    std::vector<ContractDev> cons;
    std::vector<uint32_t> item_idx;  // arithmetic items: start of each contract's items (launch order), then order
    std::vector<StaticDev> statics;  // per contract, static-schedule launches
    uint64_t total = 0, path_steps = 0, item_paths = 0, n_items = 0;
    uint32_t slots = 0, surv_base = 0;
    size_t smem = 0;
    const void *kfn = nullptr;
    int grid_blocks = 0;
};

// Device buffers a plan's tables are uploaded to (counters: 64 zeroed bytes;
// items: the plan's item_idx).
struct PathBuffers {
    void *progs, *steps, *disc, *cons, *thr, *items;
    uint32_t *counters;
    double *pv;
    void *statics;
};

// Lays out the tables of `jobs` (sets each job's pv offset) and the launch
// geometry; item_paths = 0 picks the default work-item size; pair = true
// launches the coarse kernels of multilevel pairs (k_paths, _PAIR models).
PathPlan plan_paths(std::vector<Job> &jobs, const kx_mc_config &cfg, int ns, int minb, bool lean,
                    uint64_t item_paths, bool stat, bool pair = false);
PathArgs path_args(const PathPlan &P, const PathBuffers &B);
void upload_plan(const PathPlan &P, const PathBuffers &B, cudaStream_t s);
size_t plan_upload_bytes(const PathPlan &P);

// Prices a correlated multi-factor job with k_multi_lean when its contract
// has affine conditions and amounts on a static schedule (per-path values at
// c.pv[0 .. n_paths)); false, with nothing launched, otherwise.
bool multi_lean_run(Ctx &c, Job &j, const kx_mc_config &cfg);

// The fine and coarse paths of multilevel runs in one k_mlmc_pairs launch when
// every job has a static schedule (fine[q] is run q; coarse[] the runs of
// level >= 1 in order). Per-path values go to c.mlmc: the fine paths of all
// runs from 0 (nfine in total), the coarse ones from nfine; the jobs' pv_off
// are set to those offsets. False, with nothing launched, otherwise.
bool mlmc_pairs_run(Ctx &c, std::vector<Job> &fine, std::vector<Job> &coarse, const kx_mc_config &cfg,
                    uint64_t &nfine);

// Raises the error the device error word of a path launch reports.
void check_err_word(uint32_t err);

// Merge of consecutive chunk statistics in chunk order (Chan et al.).
Stats merge_chunks(const ChunkOut *h, size_t n);
// One launch of the chunk statistics of prices: chunk q of `chunks` reduces
// values[begin + i] into out[q] (exact integer sums, chunk_moments_exact).
void launch_chunk_stats(cudaStream_t s, const double *values, const ChunkDesc *chunks, ChunkOut *out,
                        unsigned n_chunks);

// Per-call bookkeeping of the launch statistics.
void begin_call(Ctx &c);
void end_call(Ctx &c);

}  // namespace kx
