// batch.cu — price_batch_gbm (src/pricer.rs:250-294): every contract of a
// book valued on ONE shared simulation of the merged grid.
//
// Contracts whose when/anytime/until conditions depend on time only have a
// path-independent flow schedule (which flow is paid at which grid step).
// For those, k_flows simulates each path once and, at every step that has
// flows, evaluates the amounts of all contracts paid there and adds them to
// the contract's per-path value: one simulation serves the whole book, as in
// the reference. Common amounts (call / put on the spot) are recognised on the
// host and evaluated inline; anything else runs the expression interpreter.
// Contracts with price-dependent conditions or averages go through the
// general path kernel on the same grid and seed (hence the same normals and
// the same simulated paths).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "device_common.cuh"
#include "engine.hpp"
#include "paths_kernel.cuh"

namespace kx {

enum FlowKind : int { FK_CONST = 0, FK_CALL = 1, FK_PUT = 2, FK_GENERAL = 3 };

struct FlowRec {
    int contract;   // output row
    int kind;       // FlowKind
    int prog;       // program (FK_GENERAL)
    int code_off, code_len;
    int only;       // the contract's only flow: its value is stored, not added
    double a;       // strike (FK_CALL / FK_PUT)
    double sign;    // +1 / -1 (FK_CONST: the amount)
    float af, signf;  // the same in FP32 (no conversion on the FP64 pipe per path)
};

struct FlowArgs {
    const KxProgram *progs;
    const FlowRec *flows;
    const int *first;      // flows of step k: [first[k], first[k + 1])
    const int *next;       // next[k]: first step >= k with flows (n_times: none)
    const void *steps;     // StepRec<Real>
    const double *disc;
    int n_times;
    int n_contracts;
    uint64_t n_paths, seed;
    int model, scheme;
    double s0, v0, kappa, theta, sigma_v, rho, rho_perp, r;
    const double *z64;
    const float *z32;
    uint64_t z_dpp;
    double *pv;            // [n_contracts][n_paths], zeroed before the launch
};

template <class Real>
__device__ __forceinline__ Real flow_a(const FlowRec &F) { return sizeof(Real) == 4 ? (Real)F.af : (Real)F.a; }
template <class Real>
__device__ __forceinline__ Real flow_sign(const FlowRec &F) { return sizeof(Real) == 4 ? (Real)F.signf : (Real)F.sign; }

template <class Real>
__device__ __forceinline__ void pay_flows(const FlowArgs &A, int k, Real S, uint64_t path) {
    const double df = A.disc[k];
    for (int f = A.first[k]; f < A.first[k + 1]; ++f) {
        const FlowRec &F = A.flows[f];
        Real amt;
        if (F.kind == FK_CALL) amt = flow_sign<Real>(F) * fmax(S - flow_a<Real>(F), Real(0));
        else if (F.kind == FK_PUT) amt = flow_sign<Real>(F) * fmax(flow_a<Real>(F) - S, Real(0));
        else if (F.kind == FK_CONST) amt = flow_sign<Real>(F);
        else {
            uint32_t e = 0;
            amt = eval_code<Real>(A.progs[F.prog], F.code_off, F.code_len, AccView<Real>{nullptr, 0}, 0u, k, S, e);
        }
        double &dst = A.pv[(uint64_t)F.contract * A.n_paths + path];
        if (F.only) dst = (double)amt * df;
        else dst += (double)amt * df;
    }
}

template <class Real, int MODEL>
__global__ void __launch_bounds__(256) k_flows(const FlowArgs A) {
    constexpr int DRAWS = MODEL == KX_MODEL_GBM ? 1 : 2;
    const StepRec<Real> *R = reinterpret_cast<const StepRec<Real> *>(A.steps);
    const Real s0 = (Real)A.s0, r = (Real)A.r, kap = (Real)A.kappa, th = (Real)A.theta, sv = (Real)A.sigma_v,
               rho = (Real)A.rho, rp = (Real)A.rho_perp;
    for (uint64_t path = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; path < A.n_paths;
         path += (uint64_t)gridDim.x * blockDim.x) {
        Real y = Real(0), v = (Real)fmax(A.v0, 0.0);
        int nf = A.next[0];
        if (nf == 0) {
            pay_flows<Real>(A, 0, s0, path);
            nf = A.next[1];
        }
        // one Philox block (4 normals) per SPB steps, walked with compile-time indices
        constexpr int SPB = 4 / DRAWS;
        for (int k = 1; k < A.n_times; k += SPB) {
            const uint64_t d = (uint64_t)(k - 1) * DRAWS;
            Real z[4];
            if (A.z64 == nullptr && A.z32 == nullptr) {
                const uint4 w = philox4x32_10(make_uint4((uint32_t)(d >> 2), (uint32_t)path, (uint32_t)(path >> 32), 0u),
                                              (uint32_t)A.seed, (uint32_t)(A.seed >> 32));
                box_muller(w.x, w.y, z[0], z[1]);
                box_muller(w.z, w.w, z[2], z[3]);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    z[j] = d + j < A.z_dpp ? (A.z64 ? (Real)A.z64[path * A.z_dpp + d + j] : (Real)A.z32[path * A.z_dpp + d + j])
                                           : Real(0);
            }
#pragma unroll
            for (int j = 0; j < SPB; ++j) {
                const int kk = k + j;
                if (kk >= A.n_times) break;
                const StepRec<Real> rec = R[kk];
                if (MODEL == KX_MODEL_GBM) y = gbm_step(y, rec.c0, rec.c1, z[j]);
                else heston_step<Real>(r, kap, th, sv, rho, rp, A.scheme, rec.c0, rec.c1, z[2 * j], z[2 * j + 1], y, v);
                if (kk == nf) {
                    pay_flows<Real>(A, kk, spot_of<Real>(s0, y), path);
                    nf = A.next[kk + 1];
                }
            }
        }
    }
}

// Amount kind of a flow slot from its lowered code (host).
static FlowRec classify(const KxProgram &P, int leaf) {
    const KxLeaf &L = P.leaf[leaf];
    FlowRec f{};
    f.sign = 1.0;
    if (L.kind == AK_CONST) {
        f.kind = FK_CONST;
        f.sign = L.sign;
        return f;
    }
    f.kind = FK_GENERAL;
    f.code_off = L.code_off;
    f.code_len = L.code_len;
    const KxIns *c = P.code + L.code_off;
    int n = L.code_len;
    double sign = 1.0;
    if (n == 6 && c[5].op == OP_NEG) {
        sign = -1.0;
        n = 5;
    }
    if (n == 5 && c[2].op == OP_SUB && c[3].op == OP_CONST && P.cpool[c[3].arg] == 0.0 && c[4].op == OP_MAX) {
        if (c[0].op == OP_SPOT && c[1].op == OP_CONST) {
            f.kind = FK_CALL;
            f.a = P.cpool[c[1].arg];
            f.sign = sign;
        } else if (c[0].op == OP_CONST && c[1].op == OP_SPOT) {
            f.kind = FK_PUT;
            f.a = P.cpool[c[0].arg];
            f.sign = sign;
        }
    }
    return f;
}

template <class Real, int MODEL>
static const void *flows_kernel() {
    return reinterpret_cast<const void *>(&k_flows<Real, MODEL>);
}

}  // namespace kx

using namespace kx;

extern "C" kx_status kx_price_batch_shared(size_t n, const kx_program *const *progs, const kx_model *model,
                                           const kx_mc_config *cfg, kx_price_result *out) {
    return guarded([&] {
        if (n == 0) return;  // pricer.rs:255-257
        if (!progs || !out || !cfg) raise(KX_INVALID_ARGUMENT, "NULL array");
        Model m = model_from_c(model);
        if (cfg->rng != KX_RNG_PHILOX && cfg->rng != KX_RNG_SHARED_DRAWS) raise(KX_INVALID_ARGUMENT, "unknown rng");
        if (cfg->precision != KX_PREC_FP32 && cfg->precision != KX_PREC_FP64) raise(KX_INVALID_ARGUMENT, "unknown precision");
        if (cfg->flags != 0) raise(KX_INVALID_ARGUMENT, "flags must be 0");
        if (cfg->n_paths >= (1ull << 32)) raise(KX_INVALID_ARGUMENT, "n_paths must be below 2^32");
        validate_model(m);
        // merged plan (pricer.rs:260-279)
        Plan merged;
        for (size_t i = 0; i < n; ++i) {
            const Program &p = program_of(progs[i]);
            merged.fixed_dates.insert(merged.fixed_dates.end(), p.plan.fixed_dates.begin(), p.plan.fixed_dates.end());
            merged.horizon = std::max(merged.horizon, p.plan.horizon);
            merged.needs_fine_grid = merged.needs_fine_grid || p.plan.needs_fine_grid;
        }
        auto grid = time_grid_forced(merged, cfg->steps_per_year, m.requires_fine_grid());
        validate_grid(grid);
        const int nt = (int)grid.size();
        const uint64_t np = cfg->n_paths;
        const bool f64 = cfg->precision == KX_PREC_FP64;
        // split: static schedules share one simulation, the rest use the path kernel
        std::vector<KxProgram> bound(n);
        std::vector<StepTables> tabs(n);
        std::vector<size_t> stat, dyn;
        std::vector<StaticSchedule> sched(n);
        for (size_t i = 0; i < n; ++i) {
            const Program &p = program_of(progs[i]);
            bind(p.low, grid, m, cfg->rate, bound[i], tabs[i]);
            sched[i] = static_schedule(bound[i], tabs[i]);
            bool ok = sched[i].static_ok && bound[i].n_acc == 0;
            for (auto &f : sched[i].flows) ok = ok && f.price_untils == 0;
            (ok ? stat : dyn).push_back(i);
        }
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        std::vector<Stats> st_all(n);
        if (!stat.empty()) {
            std::vector<std::vector<FlowRec>> at(nt);
            std::vector<KxProgram> progs_s;
            for (size_t q = 0; q < stat.size(); ++q) {
                const size_t i = stat[q];
                progs_s.push_back(bound[i]);
                for (auto &f : sched[i].flows) {
                    FlowRec r = classify(bound[i], f.leaf);
                    r.contract = (int)q;
                    r.prog = (int)q;
                    r.only = sched[i].flows.size() == 1 ? 1 : 0;
                    r.af = (float)r.a;
                    r.signf = (float)r.sign;
                    at[f.step].push_back(r);
                }
            }
            std::vector<FlowRec> flows;
            std::vector<int> first(nt + 1), next(nt + 1);
            for (int k = 0; k < nt; ++k) {
                first[k] = (int)flows.size();
                flows.insert(flows.end(), at[k].begin(), at[k].end());
            }
            first[nt] = (int)flows.size();
            next[nt] = nt;
            for (int k = nt - 1; k >= 0; --k) next[k] = first[k + 1] > first[k] ? k : next[k + 1];
            std::vector<unsigned char> steps(nt * (f64 ? sizeof(StepRec<double>) : sizeof(StepRec<float>)));
            for (int k = 0; k < nt; ++k) {
                if (f64) reinterpret_cast<StepRec<double> *>(steps.data())[k] = {tabs[stat[0]].c0[k], tabs[stat[0]].c1[k], 0u, 0u};
                else reinterpret_cast<StepRec<float> *>(steps.data())[k] = {(float)tabs[stat[0]].c0[k], (float)tabs[stat[0]].c1[k], 0u, 0u};
            }
            const size_t ns = stat.size();
            c.progs.ensure(progs_s.size() * sizeof(KxProgram));
            c.items.ensure(std::max<size_t>(1, flows.size()) * sizeof(FlowRec));
            c.misc.ensure(2 * (nt + 1) * sizeof(int));
            c.steps.ensure(steps.size());
            c.disc.ensure(nt * sizeof(double));
            c.pv.ensure(std::max<uint64_t>(1, np * ns) * sizeof(double));
            KX_CUDA(cudaMemcpyAsync(c.progs.p, progs_s.data(), progs_s.size() * sizeof(KxProgram), cudaMemcpyHostToDevice, c.stream));
            if (!flows.empty())
                KX_CUDA(cudaMemcpyAsync(c.items.p, flows.data(), flows.size() * sizeof(FlowRec), cudaMemcpyHostToDevice, c.stream));
            KX_CUDA(cudaMemcpyAsync(c.misc.p, first.data(), (nt + 1) * sizeof(int), cudaMemcpyHostToDevice, c.stream));
            KX_CUDA(cudaMemcpyAsync(c.misc.as<int>() + nt + 1, next.data(), (nt + 1) * sizeof(int), cudaMemcpyHostToDevice, c.stream));
            KX_CUDA(cudaMemcpyAsync(c.steps.p, steps.data(), steps.size(), cudaMemcpyHostToDevice, c.stream));
            KX_CUDA(cudaMemcpyAsync(c.disc.p, tabs[stat[0]].disc.data(), nt * sizeof(double), cudaMemcpyHostToDevice, c.stream));
            // rows of contracts with several flows (or none) are added to: zero them; a contract
            // with a single flow has it stored on every path (every path walks every step)
            bool all_single = true;
            for (size_t q = 0; q < stat.size(); ++q) all_single = all_single && sched[stat[q]].flows.size() == 1;
            if (!all_single)
                KX_CUDA(cudaMemsetAsync(c.pv.p, 0, std::max<uint64_t>(1, np * ns) * sizeof(double), c.stream));
            FlowArgs a{};
            a.progs = c.progs.as<KxProgram>();
            a.flows = c.items.as<FlowRec>();
            a.first = c.misc.as<int>();
            a.next = c.misc.as<int>() + nt + 1;
            a.steps = c.steps.p;
            a.disc = c.disc.as<double>();
            a.n_times = nt;
            a.n_contracts = (int)ns;
            a.n_paths = np;
            a.seed = cfg->seed;
            a.model = m.kind;
            a.scheme = m.scheme;
            a.s0 = m.s0;
            a.v0 = m.v0; a.kappa = m.kappa; a.theta = m.theta; a.sigma_v = m.sigma_v; a.rho = m.rho;
            a.rho_perp = std::sqrt(std::max(1.0 - m.rho * m.rho, 0.0));
            a.r = m.r;
            if (cfg->rng == KX_RNG_SHARED_DRAWS) {
                DrawStore &ds = c.draws;
                if (!ds.set) raise(KX_INVALID_ARGUMENT, "no shared draws registered");
                if (ds.n_paths < np || ds.dpp < (uint64_t)(nt - 1) * m.draws_per_step())
                    raise(KX_INVALID_ARGUMENT, "shared draws too small for this simulation");
                a.z64 = ds.is64 ? ds.z64.as<double>() : nullptr;
                a.z32 = ds.is64 ? nullptr : ds.z32.as<float>();
                a.z_dpp = ds.dpp;
            }
            a.pv = c.pv.as<double>();
            const void *kfn = m.kind == KX_MODEL_GBM ? (f64 ? flows_kernel<double, KX_MODEL_GBM>() : flows_kernel<float, KX_MODEL_GBM>())
                                                     : (f64 ? flows_kernel<double, KX_MODEL_HESTON>() : flows_kernel<float, KX_MODEL_HESTON>());
            if (np > 0) {
                const int full = persistent_blocks(kfn, 256, 0);
                const int blocks = (int)std::min<uint64_t>((uint64_t)full, (np + 255) / 256);
                void *args[] = {&a};
                KX_CUDA(cudaEventRecord(c.ev0, c.stream));
                KX_CUDA(cudaLaunchKernel(kfn, dim3(blocks), dim3(256), args, 0, c.stream));
                KX_CUDA(cudaEventRecord(c.ev1, c.stream));
                KX_CUDA(cudaEventSynchronize(c.ev1));
                float ms = 0.f;
                KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
                c.last.kernel_ms += ms;
                c.last.kernel_launches++;
            }
            c.last.path_steps += np * (uint64_t)(nt - 1);
            c.last.steps_simulated += np * (uint64_t)(nt - 1);
            std::vector<StatsJob> sj(ns);
            for (size_t q = 0; q < ns; ++q) {
                sj[q].begin = (uint64_t)q * np;
                sj[q].n = np;
            }
            auto st = device_stats(c, c.pv.as<double>(), 0, sj);
            for (size_t q = 0; q < ns; ++q) st_all[stat[q]] = st[q];
        }
        if (!dyn.empty()) {  // same grid and seed: the same simulated paths
            std::vector<const Program *> dp;
            for (size_t i : dyn) dp.push_back(&program_of(progs[i]));
            auto st = batch_paths(c, dp, m, *cfg, grid);
            for (size_t q = 0; q < dyn.size(); ++q) st_all[dyn[q]] = st[q];
        }
        for (size_t i = 0; i < n; ++i) out[i] = finish(st_all[i]);
        c.last.total_ms += now_ms();
    });
}
