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

// ---------------------------------------------------------------------------
// Pathwise sensitivities of a book of European flows on the shared simulation
// (kx_price_batch_sens). Every contract pays one closed-form amount A(S) at a
// time-only date t, so its derivative in a parameter p is
// df * A'(S) * S * dy_t/dp (y the log-spot): the derivatives of y and of the
// variance v in each parameter are carried forward along the path (tangent
// mode), and every contract paid at a step takes them from there. For many
// contracts on one simulation this replaces one reverse sweep per contract
// (kx_greeks_adjoint) by a single forward pass; the derivative is the same
// pathwise one, term for term (the reverse sweep of adjoint.cu transposed):
//   GBM:    dy/dsigma += -sigma dt + sqrt(dt) z;                 dy/dr = t
//   Heston: vp = max(v, 0) (full truncation) or v, m = 0 where the truncation
//           bites, sqv = sqrt(vp), mix = rho z1 + rho_perp z2:
//           dy' = dy + (-dt/2 + z1 sq / (2 sqv)) m dv
//           dv' = keep * ((1 + (-kappa dt + sigma_v mix sq / (2 sqv)) m) dv + c_p)
//           c_v0 = 0, c_kappa = (theta - vp) dt, c_theta = kappa dt,
//           c_sigma_v = sqv mix sq, c_rho = sigma_v sqv (z1 + drho_perp/drho z2) sq,
//           keep = 0 where the reference scheme's floor bit (v' = 0), dv_0/dv0 = 1.
// Outputs per contract and path (doubles), [q][contract][path]: q = 0 d/ds0
// (dS/ds0 = S/s0), 1 d/dr (drift dy/dr = t and the discount, t (g - A df), as
// greeks.rs:70 moves both), then GBM d/dsigma | Heston d/dv0, d/dkappa,
// d/dtheta, d/dsigma_v, d/drho, each formed in the path precision. The FP32
// kernel reads FP32 copies of every parameter and table (GB300's FP64 pipe
// is slow: no conversion per step); per flow only the price, as in k_flows,
// and the outputs' conversions touch FP64.
// ---------------------------------------------------------------------------
struct SensArgs {
    FlowArgs F;              // the simulation and its flows; F.pv: the prices
    const double *times;     // grid times
    const void *dtq;         // StepRec<Real> {dt, sqrt(dt)} of every step (GBM's volatility tangent)
    const float *discf, *timesf;  // FP32 copies of the discount factors and the grid times
    double *dv;              // [2 + NP][contract][path]
    double inv_s0, sigma, drp;
    // FP32 copies: s0, r, kappa, theta, sigma_v, rho, rho_perp, drp, sigma, 1 / s0
    float pf[10];
};

template <class Real>
__device__ __forceinline__ Real sens_par(const SensArgs &S, double d, int i) {
    return sizeof(Real) == 4 ? (Real)S.pf[i] : (Real)d;
}

template <class Real, int NP>
__device__ __forceinline__ void pay_flows_sens(const SensArgs &S, int k, Real Sk, const Real (&ty)[NP], uint64_t path,
                                               Real inv_s0) {
    const FlowArgs &A = S.F;
    const double df = A.disc[k];
    const Real dfr = sizeof(Real) == 4 ? (Real)S.discf[k] : (Real)df,
               tk = sizeof(Real) == 4 ? (Real)S.timesf[k] : (Real)S.times[k];
    const uint64_t np = A.n_paths, rows = (uint64_t)A.n_contracts * np;
    for (int f = A.first[k]; f < A.first[k + 1]; ++f) {
        const FlowRec &F = A.flows[f];
        const Real sg = flow_sign<Real>(F), K = flow_a<Real>(F);
        Real amt, damt;  // the amount and its derivative in the spot
        if (F.kind == FK_CALL) {
            amt = sg * fmax(Sk - K, Real(0));
            damt = Sk > K ? sg : Real(0);
        } else if (F.kind == FK_PUT) {
            amt = sg * fmax(K - Sk, Real(0));
            damt = K > Sk ? -sg : Real(0);
        } else {
            amt = sg;
            damt = Real(0);
        }
        const double pv = (double)amt * df;
        const uint64_t o = (uint64_t)F.contract * np + path;
        A.pv[o] = pv;
        const Real g = damt * Sk * dfr;  // d pv / d y
        S.dv[o] = (double)(g * inv_s0);
        S.dv[rows + o] = (double)(tk * (g - amt * dfr));
#pragma unroll
        for (int p = 0; p < NP; ++p) S.dv[(2 + p) * rows + o] = (double)(g * ty[p]);
    }
}

template <class Real, int MODEL>
__global__ void __launch_bounds__(256, sizeof(Real) == 4 ? 4 : 2) k_flows_sens(const SensArgs S) {
    const FlowArgs &A = S.F;
    constexpr bool HESTON = MODEL == KX_MODEL_HESTON;
    constexpr int DRAWS = HESTON ? 2 : 1, NP = HESTON ? 5 : 1;
    const StepRec<Real> *R = reinterpret_cast<const StepRec<Real> *>(A.steps);
    const StepRec<Real> *Q = reinterpret_cast<const StepRec<Real> *>(S.dtq);
    const Real s0 = sens_par<Real>(S, A.s0, 0), r = sens_par<Real>(S, A.r, 1), kap = sens_par<Real>(S, A.kappa, 2),
               th = sens_par<Real>(S, A.theta, 3), sv = sens_par<Real>(S, A.sigma_v, 4),
               rho = sens_par<Real>(S, A.rho, 5), rp = sens_par<Real>(S, A.rho_perp, 6),
               drp = sens_par<Real>(S, S.drp, 7), sig = sens_par<Real>(S, S.sigma, 8),
               inv_s0 = sens_par<Real>(S, S.inv_s0, 9);
    const bool ft = A.scheme == KX_HESTON_FULL_TRUNCATION;
    for (uint64_t path = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; path < A.n_paths;
         path += (uint64_t)gridDim.x * blockDim.x) {
        Real y = Real(0), v = (Real)fmax(A.v0, 0.0);
        Real ty[NP], tv[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) ty[p] = tv[p] = Real(0);
        if (HESTON) tv[0] = A.v0 > 0.0 ? Real(1) : Real(0);  // dv_0 / dv0
        int nf = A.next[0];
        if (nf == 0) {
            pay_flows_sens<Real, NP>(S, 0, s0, ty, path, inv_s0);
            nf = A.next[1];
        }
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
                if (!HESTON) {
                    const StepRec<Real> q = Q[kk];
                    ty[0] += -sig * q.c0 + q.c1 * z[j];
                    y = gbm_step(y, rec.c0, rec.c1, z[j]);
                } else {
                    const Real z1 = z[2 * j], z2 = z[2 * j + 1], dt = rec.c0, sq = rec.c1;
                    const Real vp = ft ? fmax(v, Real(0)) : v;
                    const Real m = (ft && v <= Real(0)) ? Real(0) : Real(1);
                    const Real sqv = sqrt(vp);
                    const Real dsq = sqv > Real(0) ? Real(0.5) / sqv : Real(0);
                    const Real mix = rho * z1 + rp * z2;
                    const Real dx_dv = (Real(-0.5) * dt + z1 * sq * dsq) * m;
                    const Real dvn_dv = Real(1) + (-kap * dt + sv * mix * sq * dsq) * m;
                    const Real cp[5] = {Real(0), (th - vp) * dt, kap * dt, sqv * mix * sq,
                                        sv * sqv * (z1 + drp * z2) * sq};
                    heston_step<Real>(r, kap, th, sv, rho, rp, A.scheme, dt, sq, z1, z2, y, v);
                    const Real keep = (ft || v > Real(0)) ? Real(1) : Real(0);
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        ty[p] += dx_dv * tv[p];
                        tv[p] = keep * (dvn_dv * tv[p] + cp[p]);
                    }
                }
                if (kk == nf) {
                    pay_flows_sens<Real, NP>(S, kk, spot_of<Real>(s0, y), ty, path, inv_s0);
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
    if ((n == 1 || (n == 2 && c[1].op == OP_NEG)) && c[0].op == OP_CONST) {  // a constant amount as code
        f.kind = FK_CONST;
        f.sign = n == 2 ? -P.cpool[c[0].arg] : P.cpool[c[0].arg];
        return f;
    }
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

// A book on one shared simulation (price_batch_gbm, pricer.rs:250-294): the
// merged grid, each contract bound to it, and the split into contracts with
// static flow schedules (valued on the shared simulation by k_flows) and the
// rest (the general path kernel on the same grid and seed).
struct SharedBook {
    Model m;
    std::vector<double> grid;
    std::vector<KxProgram> bound;
    std::vector<StepTables> tabs;
    std::vector<StaticSchedule> sched;
    std::vector<size_t> stat, dyn;
};

static SharedBook shared_book(size_t n, const kx_program *const *progs, const kx_model *model,
                              const kx_mc_config *cfg) {
    SharedBook B;
    B.m = model_from_c(model);
    if (cfg->rng != KX_RNG_PHILOX && cfg->rng != KX_RNG_SHARED_DRAWS) raise(KX_INVALID_ARGUMENT, "unknown rng");
    if (cfg->precision != KX_PREC_FP32 && cfg->precision != KX_PREC_FP64) raise(KX_INVALID_ARGUMENT, "unknown precision");
    if (cfg->flags != 0) raise(KX_INVALID_ARGUMENT, "flags must be 0");
    if (cfg->n_paths >= (1ull << 32)) raise(KX_INVALID_ARGUMENT, "n_paths must be below 2^32");
    validate_model(B.m);
    // merged plan (pricer.rs:260-279)
    Plan merged;
    for (size_t i = 0; i < n; ++i) {
        const Program &p = program_of(progs[i]);
        merged.fixed_dates.insert(merged.fixed_dates.end(), p.plan.fixed_dates.begin(), p.plan.fixed_dates.end());
        merged.horizon = std::max(merged.horizon, p.plan.horizon);
        merged.needs_fine_grid = merged.needs_fine_grid || p.plan.needs_fine_grid;
    }
    B.grid = time_grid_forced(merged, cfg->steps_per_year, B.m.requires_fine_grid());
    validate_grid(B.grid);
    // split: static schedules share one simulation, the rest use the path kernel
    B.bound.resize(n);
    B.tabs.resize(n);
    B.sched.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const Program &p = program_of(progs[i]);
        bind(p.low, B.grid, B.m, cfg->rate, B.bound[i], B.tabs[i]);
        B.sched[i] = static_schedule(B.bound[i], B.tabs[i]);
        bool ok = B.sched[i].static_ok && B.bound[i].n_acc == 0;
        for (auto &f : B.sched[i].flows) ok = ok && f.price_untils == 0;
        (ok ? B.stat : B.dyn).push_back(i);
    }
    return B;
}

// The flows of the static contracts by step: the flows paid at step k are
// flows[first[k] .. first[k + 1]), next[k] the first step >= k with flows.
struct FlowTable {
    std::vector<KxProgram> progs;
    std::vector<FlowRec> flows;
    std::vector<int> first, next;
    bool all_single = true;  // every contract has exactly one flow
};

static FlowTable flow_table(const SharedBook &B) {
    const int nt = (int)B.grid.size();
    FlowTable T;
    std::vector<std::vector<FlowRec>> at(nt);
    for (size_t q = 0; q < B.stat.size(); ++q) {
        const size_t i = B.stat[q];
        T.progs.push_back(B.bound[i]);
        for (auto &f : B.sched[i].flows) {
            FlowRec r = classify(B.bound[i], f.leaf);
            r.contract = (int)q;
            r.prog = (int)q;
            r.only = B.sched[i].flows.size() == 1 ? 1 : 0;
            r.af = (float)r.a;
            r.signf = (float)r.sign;
            at[f.step].push_back(r);
        }
        T.all_single = T.all_single && B.sched[i].flows.size() == 1;
    }
    T.first.resize(nt + 1);
    T.next.resize(nt + 1);
    for (int k = 0; k < nt; ++k) {
        T.first[k] = (int)T.flows.size();
        T.flows.insert(T.flows.end(), at[k].begin(), at[k].end());
    }
    T.first[nt] = (int)T.flows.size();
    T.next[nt] = nt;
    for (int k = nt - 1; k >= 0; --k) T.next[k] = T.first[k + 1] > T.first[k] ? k : T.next[k + 1];
    return T;
}

// Uploads the flow table, the steps and the discount factors of the shared
// simulation to the context's buffers and returns the kernel arguments
// (prices of contract q at pv[q * n_paths + path], c.pv).
static FlowArgs upload_flows(Ctx &c, const SharedBook &B, const FlowTable &T, const kx_mc_config &cfg) {
    const int nt = (int)B.grid.size();
    const uint64_t np = cfg.n_paths;
    const bool f64 = cfg.precision == KX_PREC_FP64;
    const Model &m = B.m;
    const StepTables &tab = B.tabs[B.stat[0]];
    std::vector<unsigned char> steps(nt * (f64 ? sizeof(StepRec<double>) : sizeof(StepRec<float>)));
    for (int k = 0; k < nt; ++k) {
        if (f64) reinterpret_cast<StepRec<double> *>(steps.data())[k] = {tab.c0[k], tab.c1[k], 0u, 0u};
        else reinterpret_cast<StepRec<float> *>(steps.data())[k] = {(float)tab.c0[k], (float)tab.c1[k], 0u, 0u};
    }
    const size_t ns = B.stat.size();
    c.progs.ensure(T.progs.size() * sizeof(KxProgram));
    c.items.ensure(std::max<size_t>(1, T.flows.size()) * sizeof(FlowRec));
    c.misc.ensure(2 * (nt + 1) * sizeof(int));
    c.steps.ensure(steps.size());
    c.disc.ensure(nt * sizeof(double));
    c.pv.ensure(std::max<uint64_t>(1, np * ns) * sizeof(double));
    KX_CUDA(cudaMemcpyAsync(c.progs.p, T.progs.data(), T.progs.size() * sizeof(KxProgram), cudaMemcpyHostToDevice,
                            c.stream));
    if (!T.flows.empty())
        KX_CUDA(cudaMemcpyAsync(c.items.p, T.flows.data(), T.flows.size() * sizeof(FlowRec), cudaMemcpyHostToDevice,
                                c.stream));
    KX_CUDA(cudaMemcpyAsync(c.misc.p, T.first.data(), (nt + 1) * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemcpyAsync(c.misc.as<int>() + nt + 1, T.next.data(), (nt + 1) * sizeof(int), cudaMemcpyHostToDevice,
                            c.stream));
    KX_CUDA(cudaMemcpyAsync(c.steps.p, steps.data(), steps.size(), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemcpyAsync(c.disc.p, tab.disc.data(), nt * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    // rows of contracts with several flows (or none) are added to: zero them; a contract
    // with a single flow has it stored on every path (every path walks every step)
    if (!T.all_single) KX_CUDA(cudaMemsetAsync(c.pv.p, 0, std::max<uint64_t>(1, np * ns) * sizeof(double), c.stream));
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
    a.seed = cfg.seed;
    a.model = m.kind;
    a.scheme = m.scheme;
    a.s0 = m.s0;
    a.v0 = m.v0;
    a.kappa = m.kappa;
    a.theta = m.theta;
    a.sigma_v = m.sigma_v;
    a.rho = m.rho;
    a.rho_perp = std::sqrt(std::max(1.0 - m.rho * m.rho, 0.0));
    a.r = m.r;
    if (cfg.rng == KX_RNG_SHARED_DRAWS) {
        DrawStore &ds = c.draws;
        if (!ds.set) raise(KX_INVALID_ARGUMENT, "no shared draws registered");
        if (ds.n_paths < np || ds.dpp < (uint64_t)(nt - 1) * m.draws_per_step())
            raise(KX_INVALID_ARGUMENT, "shared draws too small for this simulation");
        a.z64 = ds.is64 ? ds.z64.as<double>() : nullptr;
        a.z32 = ds.is64 ? nullptr : ds.z32.as<float>();
        a.z_dpp = ds.dpp;
    }
    a.pv = c.pv.as<double>();
    return a;
}

// One launch of a shared-simulation kernel over np paths, timed into c.last.
static void launch_shared(Ctx &c, const void *kfn, void *arg, uint64_t np) {
    if (np == 0) return;
    const int full = persistent_blocks(kfn, 256, 0);
    const int blocks = (int)std::min<uint64_t>((uint64_t)full, (np + 255) / 256);
    void *args[] = {arg};
    KX_CUDA(cudaEventRecord(c.ev0, c.stream));
    KX_CUDA(cudaLaunchKernel(kfn, dim3(blocks), dim3(256), args, 0, c.stream));
    KX_CUDA(cudaEventRecord(c.ev1, c.stream));
    KX_CUDA(cudaEventSynchronize(c.ev1));
    float ms = 0.f;
    KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.last.kernel_ms += ms;
    c.last.kernel_launches++;
}

}  // namespace kx

using namespace kx;

extern "C" kx_status kx_price_batch_shared(size_t n, const kx_program *const *progs, const kx_model *model,
                                           const kx_mc_config *cfg, kx_price_result *out) {
    return guarded([&] {
        if (n == 0) return;  // pricer.rs:255-257
        if (!progs || !out || !cfg) raise(KX_INVALID_ARGUMENT, "NULL array");
        const SharedBook B = shared_book(n, progs, model, cfg);
        const Model &m = B.m;
        const int nt = (int)B.grid.size();
        const uint64_t np = cfg->n_paths;
        const bool f64 = cfg->precision == KX_PREC_FP64;
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        std::vector<Stats> st_all(n);
        if (!B.stat.empty()) {
            const FlowTable T = flow_table(B);
            FlowArgs a = upload_flows(c, B, T, *cfg);
            const size_t ns = B.stat.size();
            const void *kfn = m.kind == KX_MODEL_GBM ? (f64 ? flows_kernel<double, KX_MODEL_GBM>() : flows_kernel<float, KX_MODEL_GBM>())
                                                     : (f64 ? flows_kernel<double, KX_MODEL_HESTON>() : flows_kernel<float, KX_MODEL_HESTON>());
            launch_shared(c, kfn, &a, np);
            c.last.path_steps += np * (uint64_t)(nt - 1);
            c.last.steps_simulated += np * (uint64_t)(nt - 1);
            std::vector<StatsJob> sj(ns);
            for (size_t q = 0; q < ns; ++q) {
                sj[q].begin = (uint64_t)q * np;
                sj[q].n = np;
            }
            auto st = device_stats(c, c.pv.as<double>(), 0, sj);
            for (size_t q = 0; q < ns; ++q) st_all[B.stat[q]] = st[q];
        }
        if (!B.dyn.empty()) {  // same grid and seed: the same simulated paths
            std::vector<const Program *> dp;
            for (size_t i : B.dyn) dp.push_back(&program_of(progs[i]));
            auto st = batch_paths(c, dp, m, *cfg, B.grid);
            for (size_t q = 0; q < B.dyn.size(); ++q) st_all[B.dyn[q]] = st[q];
        }
        for (size_t i = 0; i < n; ++i) out[i] = finish(st_all[i]);
        c.last.total_ms += now_ms();
    });
}

extern "C" kx_status kx_price_batch_sens(size_t n, const kx_program *const *progs, const kx_model *model,
                                         const kx_mc_config *cfg, kx_price_result *out, kx_sens *sens) {
    return guarded([&] {
        if (n == 0) return;
        if (!progs || !out || !sens || !cfg) raise(KX_INVALID_ARGUMENT, "NULL array");
        const SharedBook B = shared_book(n, progs, model, cfg);
        const Model &m = B.m;
        if (m.kind != KX_MODEL_GBM && m.kind != KX_MODEL_HESTON) raise(KX_UNSUPPORTED, "GBM and Heston books only");
        const FlowTable T = flow_table(B);
        bool ok = B.dyn.empty() && T.all_single;
        for (auto &f : T.flows) ok = ok && f.kind != FK_GENERAL;
        if (!ok)
            raise(KX_UNSUPPORTED, "sensitivities on a shared simulation need contracts that each pay one call, put or "
                                  "constant amount at a fixed date (kx_price_portfolio prices others with sensitivities)");
        const int nt = (int)B.grid.size();
        const uint64_t np = cfg->n_paths;
        const bool f64 = cfg->precision == KX_PREC_FP64;
        const bool heston = m.kind == KX_MODEL_HESTON;
        const int nq = heston ? 7 : 3;  // derivative outputs per contract
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        SensArgs a{};
        a.F = upload_flows(c, B, T, *cfg);
        const size_t ns = B.stat.size();
        std::vector<unsigned char> dtq(nt * (f64 ? sizeof(StepRec<double>) : sizeof(StepRec<float>)));
        for (int k = 0; k < nt; ++k) {
            const double dt = k == 0 ? 0.0 : B.grid[k] - B.grid[k - 1], sq = std::sqrt(dt);  // as the adjoint's tables
            if (f64) reinterpret_cast<StepRec<double> *>(dtq.data())[k] = {dt, sq, 0u, 0u};
            else reinterpret_cast<StepRec<float> *>(dtq.data())[k] = {(float)dt, (float)sq, 0u, 0u};
        }
        // one table upload: the grid times (double), the {dt, sqrt(dt)} records, FP32 copies of the
        // discount factors and times
        const size_t b_times = (size_t)nt * sizeof(double), b_f = (size_t)nt * sizeof(float);
        std::vector<unsigned char> tabs(b_times + dtq.size() + 2 * b_f);
        memcpy(tabs.data(), B.grid.data(), b_times);
        memcpy(tabs.data() + b_times, dtq.data(), dtq.size());
        float *ff = reinterpret_cast<float *>(tabs.data() + b_times + dtq.size());
        const StepTables &tab0 = B.tabs[B.stat[0]];
        for (int k = 0; k < nt; ++k) {
            ff[k] = (float)tab0.disc[k];
            ff[nt + k] = (float)B.grid[k];
        }
        c.grid_tabs.ensure(tabs.size());
        KX_CUDA(cudaMemcpyAsync(c.grid_tabs.p, tabs.data(), tabs.size(), cudaMemcpyHostToDevice, c.stream));
        const uint64_t rows = (uint64_t)ns * np;
        c.vr.ensure(std::max<uint64_t>(1, rows * nq) * sizeof(double));
        a.times = c.grid_tabs.as<double>();
        a.dtq = c.grid_tabs.as<unsigned char>() + b_times;
        a.discf = reinterpret_cast<const float *>(c.grid_tabs.as<unsigned char>() + b_times + dtq.size());
        a.timesf = a.discf + nt;
        a.dv = c.vr.as<double>();
        a.inv_s0 = 1.0 / m.s0;
        a.sigma = m.sigma;
        a.drp = a.F.rho_perp > 0.0 ? -m.rho / a.F.rho_perp : 0.0;
        const double pd[10] = {m.s0, a.F.r, m.kappa, m.theta, m.sigma_v, m.rho, a.F.rho_perp, a.drp, a.sigma, a.inv_s0};
        for (int q = 0; q < 10; ++q) a.pf[q] = (float)pd[q];
        const void *kfn = heston ? (f64 ? (const void *)&k_flows_sens<double, KX_MODEL_HESTON>
                                        : (const void *)&k_flows_sens<float, KX_MODEL_HESTON>)
                                 : (f64 ? (const void *)&k_flows_sens<double, KX_MODEL_GBM>
                                        : (const void *)&k_flows_sens<float, KX_MODEL_GBM>);
        launch_shared(c, kfn, &a, np);
        c.last.path_steps += np * (uint64_t)(nt - 1);
        c.last.steps_simulated += np * (uint64_t)(nt - 1);
        c.last.h2d_bytes += tabs.size();
        // statistics: the prices, the derivatives
        std::vector<StatsJob> sj(ns), sr(ns * nq);
        for (size_t q = 0; q < ns; ++q) {
            sj[q].begin = (uint64_t)q * np;
            sj[q].n = np;
            for (int o = 0; o < nq; ++o) {
                sr[o * ns + q].begin = (uint64_t)o * rows + (uint64_t)q * np;
                sr[o * ns + q].n = np;
            }
        }
        const auto sp = device_stats(c, c.pv.as<double>(), 0, sj);
        const auto sv = device_stats(c, a.dv, 0, sr);
        for (size_t q = 0; q < ns; ++q) {
            const size_t i = B.stat[q];
            out[i] = finish(sp[q]);
            kx_sens &S = sens[i];
            S = kx_sens{};
            S.price = out[i].price;
            S.price_se = out[i].std_error;
            auto put = [&](const Stats &st, double &val, double &se) {
                const kx_price_result r = finish(st);
                val = r.price;
                se = r.std_error;
            };
            put(sv[q], S.d_s0, S.se_s0);
            put(sv[1 * ns + q], S.d_r, S.se_r);
            if (heston) {
                put(sv[2 * ns + q], S.d_v0, S.se_v0);
                put(sv[3 * ns + q], S.d_kappa, S.se_kappa);
                put(sv[4 * ns + q], S.d_theta, S.se_theta);
                put(sv[5 * ns + q], S.d_sigma_v, S.se_sigma_v);
                put(sv[6 * ns + q], S.d_rho, S.se_rho);
            } else {
                put(sv[2 * ns + q], S.d_sigma, S.se_sigma);
            }
        }
        c.last.total_ms += now_ms();
    });
}
