// paths_mlmc.cu — the coupled fine / coarse paths of multilevel Monte Carlo
// (simulate_level_pair, simulator.rs:321-409 for GBM and 592-690 for Heston)
// in one kernel: k_mlmc_pairs.
//
// A level-l pair is a fine path of 2^l steps and a coarse path of 2^(l-1)
// steps driven by the same normals: a coarse GBM step adds the normals of its
// two fine steps, a coarse Heston step sums the two fine (z1, z2) pairs over
// sqrt 2. The separate launches (fine paths, then coarse paths on k_lean's
// _PAIR models) draw every normal twice and hand out every path twice; here a
// thread draws each Philox block once and advances both paths with it, and
// the runs of all levels are one launch.
//
// Contracts: the static schedules of k_lean without accumulators (European
// and Bermudan payoffs, barriers on the spot, time events). Each path is
// evaluated as k_lean evaluates it (static_event at step 0, then at every step
// where the spot leaves the barrier window or an event step is reached), with
// the same arithmetic on the same normals, so the per-path values equal the
// separate launches' bit for bit.
//
// A thread takes one pair at a time (grid-stride over the pairs of all runs,
// the longest level first); both paths of a pair have fixed lengths, so the
// lanes of a warp mostly run the same number of blocks.
#include <algorithm>

#include "launch.hpp"

namespace kx {

constexpr int MP_BLOCK = 256;
constexpr int MP_MAXRUN = KX_MLMC_MAX_LEVELS + 1;

struct MlmcRun {
    uint64_t first;        // first global pair index of the run
    uint64_t n;            // pairs
    uint64_t out_f, out_c; // per-path value slots: fine path i at out_f + i, coarse at out_c + i
    int32_t nt_f, nt_c;    // grid points of the fine and coarse paths (nt_c = 0: level 0, no coarse path)
    int32_t st_f, st_c;    // StaticDev of the fine and coarse jobs
    int32_t d_f, d_c;      // first discount factor of each
    // step coefficients of the uniform grids (fine c0, c1, coarse c0, c1) in the launch
    // precision: doubles, or floats in the first 16 bytes (no FP64 conversion per path)
    union {
        double d[4];
        float f[4];
    } coef;
    uint32_t stream, pad;
    uint32_t rk[20];       // Philox round keys of the run's seed
};

struct MlmcArgs {
    const StaticDev *statics;
    const double *disc;
    double *out;
    unsigned long long *steps_done;
    uint64_t total;
    int32_t n_runs, heston, scheme, pad;
    double s0, v0, r, kappa, theta, sigma_v, rho, rho_perp;
    MlmcRun run[MP_MAXRUN];
};
static_assert(sizeof(MlmcArgs) <= 4096, "kernel parameters");

// One path of a pair: its state, its static-schedule lane and barrier window.
template <class Real>
struct PairPath {
    Real y, v, hi, lo;
    int lim, nt;
    bool done;
    SLane L;
};

// The contract at step k of path P (static_lane_event of k_lean).
template <class Real>
__device__ __forceinline__ void pair_event(const StaticDev &T, const double *D, Real s0, int k, PairPath<Real> &P) {
    static_event<Real>(T, D, s0, P.y, k, P.L);
    static_window<Real>(T, P.L.live, P.hi, P.lo);
    P.lim = P.L.e < T.n_ev ? min(T.ev_step[P.L.e], P.nt - 1) : P.nt - 1;
    if (P.L.rem == 0u || k + 1 >= P.nt) P.done = true;
}

template <class Real, bool HESTON>
__global__ void __launch_bounds__(MP_BLOCK, sizeof(Real) == 4 ? 4 : 2) k_mlmc_pairs(const __grid_constant__ MlmcArgs A) {
    constexpr int FM = HESTON ? M_HESTON : M_GBM;            // fine steps
    constexpr int CM = HESTON ? M_HESTON_PAIR : M_GBM_PAIR;  // coarse steps
    constexpr int SPF = lean_spb<FM>();                      // fine steps per Philox block
    constexpr int SPC = lean_spb<CM>();                      // coarse steps per Philox block
    const HestonPar<Real> hp{(Real)A.r, (Real)A.kappa, (Real)A.theta, (Real)A.sigma_v, (Real)A.rho,
                             (Real)A.rho_perp, A.scheme};
    const Real s0 = (Real)A.s0;
    const Real v0 = HESTON ? fmax((Real)A.v0, Real(0)) : Real(0);
    uint32_t my_steps = 0;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < A.total;
         g += (uint64_t)gridDim.x * blockDim.x) {
        int q = 0;
        while (q + 1 < A.n_runs && A.run[q + 1].first <= g) ++q;
        const MlmcRun &U = A.run[q];
        const uint32_t path = (uint32_t)(g - U.first);
        uint32_t rk[20];
#pragma unroll
        for (int i = 0; i < 20; ++i) rk[i] = U.rk[i];
        constexpr bool F32 = sizeof(Real) == 4;
        const Real c0f = F32 ? (Real)U.coef.f[0] : (Real)U.coef.d[0], c1f = F32 ? (Real)U.coef.f[1] : (Real)U.coef.d[1];
        const Real c0c = F32 ? (Real)U.coef.f[2] : (Real)U.coef.d[2], c1c = F32 ? (Real)U.coef.f[3] : (Real)U.coef.d[3];
        const StaticDev &Tf = A.statics[U.st_f];
        const StaticDev &Tc = A.statics[U.nt_c > 0 ? U.st_c : U.st_f];
        const double *Df = A.disc + U.d_f;
        const double *Dc = A.disc + U.d_c;
        // step 0 of both paths (S = s0)
        PairPath<Real> F{Real(0), v0, Real(0), Real(0), 0, U.nt_f, false, SLane{0u, Tf.all_flows, 0, 0.0}};
        PairPath<Real> Cp{Real(0), v0, Real(0), Real(0), 0, U.nt_c, U.nt_c <= 0, SLane{0u, Tc.all_flows, 0, 0.0}};
        pair_event<Real>(Tf, Df, s0, 0, F);
        if (!Cp.done) pair_event<Real>(Tc, Dc, s0, 0, Cp);
        for (uint32_t blk = 0; !(F.done && Cp.done); ++blk) {
            const uint4 w = philox4x32_10_rk(make_uint4(blk, path, 0u, U.stream), rk);
            Real zz[4];
            box_muller(w.x, w.y, zz[0], zz[1]);
            box_muller(w.z, w.w, zz[2], zz[3]);
#pragma unroll
            for (int j = 0; j < SPF; ++j) {
                const int k = (int)blk * SPF + j + 1;
                if (!F.done) {
                    lean_model_step<Real, FM>(hp, c0f, c1f, zz, j, F.y, F.v);
                    ++my_steps;
                    if (F.y >= F.hi || F.y <= F.lo || k >= F.lim) pair_event<Real>(Tf, Df, s0, k, F);
                }
            }
#pragma unroll
            for (int j = 0; j < SPC; ++j) {
                const int k = (int)blk * SPC + j + 1;
                if (!Cp.done) {
                    lean_model_step<Real, CM>(hp, c0c, c1c, zz, j, Cp.y, Cp.v);
                    ++my_steps;
                    if (Cp.y >= Cp.hi || Cp.y <= Cp.lo || k >= Cp.lim) pair_event<Real>(Tc, Dc, s0, k, Cp);
                }
            }
        }
        A.out[U.out_f + path] = F.L.pv;
        if (U.nt_c > 0) A.out[U.out_c + path] = Cp.L.pv;
    }
    unsigned long long tot = (unsigned long long)my_steps;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(A.steps_done, tot);
}

template __global__ void k_mlmc_pairs<float, false>(const __grid_constant__ MlmcArgs);
template __global__ void k_mlmc_pairs<double, false>(const __grid_constant__ MlmcArgs);
template __global__ void k_mlmc_pairs<float, true>(const __grid_constant__ MlmcArgs);
template __global__ void k_mlmc_pairs<double, true>(const __grid_constant__ MlmcArgs);

bool mlmc_pairs_run(Ctx &c, std::vector<Job> &fine, std::vector<Job> &coarse, const kx_mc_config &cfg,
                    uint64_t &nfine) {
    const char *env = getenv("KX_PATH_KERNEL");
    if (env && (strcmp(env, "general") == 0 || strcmp(env, "lean") == 0)) return false;
    if (cfg.rng == KX_RNG_SHARED_DRAWS || fine.empty() || fine.size() > (size_t)MP_MAXRUN) return false;
    const int kind = fine[0].model.kind;
    if (kind != KX_MODEL_GBM && kind != KX_MODEL_HESTON) return false;
    // every job on a static schedule without accumulators or smoothing, on a uniform grid
    std::vector<StaticDev> statics;
    auto add = [&](const Job &j) {
        StaticDev T;
        if (j.prog.n_acc || j.dev.smooth || !j.dev.uniform || j.path_base != 0 || !build_static(j, T)) return -1;
        statics.push_back(T);
        return (int)statics.size() - 1;
    };
    MlmcArgs A;
    memset(&A, 0, sizeof A);
    const bool f64 = cfg.precision == KX_PREC_FP64;
    std::vector<double> disc;
    size_t qc = 0;
    std::vector<uint64_t> off_f(fine.size()), off_c(fine.size());
    uint64_t nf = 0, nc = 0;
    for (size_t q = 0; q < fine.size(); ++q) {
        Job &jf = fine[q];
        // the run's coarse job, in run order: level 0 (one fine step) has none
        Job *jc = nullptr;
        if (jf.dev.n_times > 2) {
            if (qc >= coarse.size()) return false;
            jc = &coarse[qc++];
        }
        off_f[q] = nf;
        nf += jf.dev.n_paths;
        if (jc) {
            off_c[q] = nc;
            nc += jc->dev.n_paths;
        }
        MlmcRun &U = A.run[q];
        U.n = jf.dev.n_paths;
        U.nt_f = jf.dev.n_times;
        if ((U.st_f = add(jf)) < 0) return false;
        U.d_f = (int32_t)disc.size();
        disc.insert(disc.end(), jf.tab.disc.begin(), jf.tab.disc.end());
        double cf[4] = {jf.dev.uc0, jf.dev.uc1, 0.0, 0.0};
        U.stream = jf.dev.stream;
        const PhiloxKeys K = philox_keys(jf.dev.seed);
        memcpy(U.rk, K.rk, sizeof U.rk);
        if (jc) {
            if (jc->dev.seed != jf.dev.seed || jc->dev.stream != jf.dev.stream || jc->dev.n_paths != jf.dev.n_paths ||
                jc->model.kind != kind)
                return false;
            U.nt_c = jc->dev.n_times;
            if ((U.st_c = add(*jc)) < 0) return false;
            U.d_c = (int32_t)disc.size();
            disc.insert(disc.end(), jc->tab.disc.begin(), jc->tab.disc.end());
            cf[2] = jc->dev.uc0;
            cf[3] = jc->dev.uc1;
        }
        for (int i = 0; i < 4; ++i) {
            if (f64) U.coef.d[i] = cf[i];
            else U.coef.f[i] = (float)cf[i];
        }
    }
    if (qc != coarse.size()) return false;
    // per-path values as the separate launches lay them out: fine paths of every run side by
    // side from 0, the coarse ones from nfine, so that a run's coarse value sits (nfine - n0)
    // after its fine one
    for (size_t q = 0, k = 0; q < fine.size(); ++q) {
        fine[q].dev.pv_off = off_f[q];
        A.run[q].out_f = off_f[q];
        if (A.run[q].nt_c > 0) {
            coarse[k].dev.pv_off = off_c[q];
            A.run[q].out_c = nf + off_c[q];
            ++k;
        }
    }
    // pairs in the launch: the longest level first
    std::vector<size_t> order(fine.size());
    for (size_t q = 0; q < order.size(); ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return A.run[a].nt_f > A.run[b].nt_f; });
    MlmcArgs B = A;
    uint64_t first = 0;
    for (size_t i = 0; i < order.size(); ++i) {
        B.run[i] = A.run[order[i]];
        B.run[i].first = first;
        first += B.run[i].n;
    }
    B.n_runs = (int32_t)fine.size();
    B.total = first;
    const Model &m = fine[0].model;
    B.heston = kind == KX_MODEL_HESTON;
    B.scheme = m.scheme;
    B.s0 = m.s0;
    const ContractDev &d = fine[0].dev;
    B.v0 = d.v0;
    B.r = d.r;
    B.kappa = d.kappa;
    B.theta = d.theta;
    B.sigma_v = d.sigma_v;
    B.rho = d.rho;
    B.rho_perp = d.rho_perp;
    nfine = nf;
    for (auto &j : fine) c.last.path_steps += j.dev.n_paths * (uint64_t)(j.dev.n_times - 1);
    for (auto &j : coarse) c.last.path_steps += j.dev.n_paths * (uint64_t)(j.dev.n_times - 1);
    c.mlmc.ensure(std::max<uint64_t>(1, 2 * nf) * sizeof(double));
    if (first == 0) return true;
    c.statics.ensure(statics.size() * sizeof(StaticDev));
    c.disc.ensure(disc.size() * sizeof(double));
    c.counters.ensure(64);
    KX_CUDA(cudaMemcpyAsync(c.statics.p, statics.data(), statics.size() * sizeof(StaticDev), cudaMemcpyHostToDevice,
                            c.stream));
    KX_CUDA(cudaMemcpyAsync(c.disc.p, disc.data(), disc.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemsetAsync(c.counters.p, 0, 64, c.stream));
    c.last.h2d_bytes += statics.size() * sizeof(StaticDev) + disc.size() * sizeof(double) + sizeof B;
    B.statics = c.statics.as<StaticDev>();
    B.disc = c.disc.as<double>();
    B.out = c.mlmc.as<double>();
    B.steps_done = c.counters.as<unsigned long long>();
    const void *kfn = f64 ? (B.heston ? (const void *)&k_mlmc_pairs<double, true> : (const void *)&k_mlmc_pairs<double, false>)
                          : (B.heston ? (const void *)&k_mlmc_pairs<float, true> : (const void *)&k_mlmc_pairs<float, false>);
    const int full = persistent_blocks(kfn, MP_BLOCK, 0);
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)full, (first + MP_BLOCK - 1) / MP_BLOCK));
    void *args[] = {&B};
    KX_CUDA(cudaEventRecord(c.ev0, c.stream));
    KX_CUDA(cudaLaunchKernel(kfn, dim3(grid), dim3(MP_BLOCK), args, 0, c.stream));
    KX_CUDA(cudaEventRecord(c.ev1, c.stream));
    c.last.kernel_launches++;
    c.last.grid_blocks = (uint32_t)grid;
    c.last.block_threads = (uint32_t)MP_BLOCK;
    c.last.path_kernel = 6u;
    unsigned long long sim = 0;
    KX_CUDA(cudaMemcpyAsync(&sim, c.counters.p, sizeof sim, cudaMemcpyDeviceToHost, c.stream));
    KX_CUDA(cudaStreamSynchronize(c.stream));
    float ms = 0.f;
    KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.last.kernel_ms += ms;
    c.last.steps_simulated += sim;
    return true;
}

}  // namespace kx
