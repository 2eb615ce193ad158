// adjoint.cu — pathwise adjoint Greeks with a reverse sweep per path.
//
// No reference counterpart: the reference only bumps and reprices
// (greeks.rs:60-98). Supported contracts are those whose payoff is a smooth
// (or smoothed) function of the path:
//   * when/anytime conditions depend on time only, so every flow date and every
//     until arming date is path-independent (the host computes that schedule);
//   * until(Spot cmp Const) barriers are replaced by a logistic survival weight
//     prod_k sigma(-+(y_k - b) / w) over the steps the until is armed, of a
//     stated width w in log-spot; time-only untils knock out deterministically;
//   * flow amounts are expressions of the spot, constants, arithmetic, max/min
//     and Average / RunningMax / RunningMin of the spot.
//
// Per path: a forward pass simulates the path (the same Philox counters as the
// pricing kernel), evaluates the smoothed payoff with forward-mode derivatives
// of each amount with respect to its inputs, and stores the state (y, v) every
// `K` steps. The reverse sweep then walks the segments backwards: each segment
// is recomputed from its checkpoint (regenerating its normals from Philox),
// and the adjoints lambda = dPV/dlog S, mu = dPV/dv are propagated through
// every step, accumulating the parameter sensitivities. Memory per path is
// (N / K + 1) states plus one K-step segment.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "device_common.cuh"
#include "engine.hpp"

namespace kx {

constexpr int ADJ_BLOCK = 128;
constexpr int ADJ_MAXF = 4;    // flows
constexpr int ADJ_MAXU = 2;    // smoothed untils
constexpr int ADJ_MAXA = 2;    // accumulators
constexpr int ADJ_MAXCK = 72;  // checkpoints
constexpr int ADJ_KMAX = 32;   // checkpoint interval
constexpr int ADJ_OUT = 9;     // per-path outputs (slot 8: price with hard barriers)

struct AdjFlow {
    int t;             // step the flow is paid at
    int kind;          // KxAmountKind
    int code_off, code_len;
    double sign;
    uint32_t su_mask;  // smoothed untils above the flow
};
struct AdjUntil {
    int arm;           // first step it weighs
    int cmp;           // KxCmp
    double thr;        // log(B / s0)
};
struct AdjAcc {
    int kind;          // KxAccKind
    int i_from, i_to;  // window (i_to: INT_MAX for running)
};

struct AdjArgs {
    const KxProgram *P;   // for the amount programs
    const void *steps;    // StepRec<Real>: GBM c0 = dt, c1 = sqrt(dt); Heston the same
    const double *disc;   // exp(-rate t_k)
    const double *times;  // t_k
    int n_times;
    int n_flows, n_su, n_acc;
    AdjFlow flow[ADJ_MAXF];
    AdjUntil su[ADJ_MAXU];
    AdjAcc acc[ADJ_MAXA];
    int K;                // checkpoint interval (multiple of 4)
    int uniform;          // every step k >= 1 has the coefficients (uc0, uc1): dt, sqrt(dt)
    double uc0, uc1;
    int model, scheme;
    uint64_t n_paths, seed;
    double s0, mu, sigma;                         // GBM (mu = drift)
    double v0, kappa, theta, sigma_v, rho, rho_perp, r;
    double inv_w;
    const double *z64;
    const float *z32;
    uint64_t z_dpp;
    uint64_t out_off;     // first output slot of this contract in each output row
};

// Forward-mode value of an amount program with derivatives with respect to
// the spot (index 0) and each accumulator (index 1 + a).
template <class Real>
struct Dual {
    Real v, d[1 + ADJ_MAXA];
};

template <class Real>
__device__ __noinline__ Dual<Real> eval_dual(const KxProgram &P, int off, int len, Real S, const Real *accv) {
    Dual<Real> st[KX_MAX_STACK];
    int sp = 0;
    for (int pc = off; pc < off + len; ++pc) {
        const KxIns ins = P.code[pc];
        Dual<Real> r;
#pragma unroll
        for (int q = 0; q < 1 + ADJ_MAXA; ++q) r.d[q] = Real(0);
        switch (ins.op) {
        case OP_CONST: r.v = (Real)P.cpool[ins.arg]; st[sp++] = r; continue;
        case OP_SPOT: r.v = S; r.d[0] = Real(1); st[sp++] = r; continue;
        case OP_ACC: r.v = accv[ins.arg]; r.d[1 + ins.arg] = Real(1); st[sp++] = r; continue;
        case OP_NEG:
            st[sp - 1].v = -st[sp - 1].v;
#pragma unroll
            for (int q = 0; q < 1 + ADJ_MAXA; ++q) st[sp - 1].d[q] = -st[sp - 1].d[q];
            continue;
        default: break;
        }
        --sp;
        const Dual<Real> a = st[sp - 1], b = st[sp];
        switch (ins.op) {
        case OP_ADD: r.v = a.v + b.v; for (int q = 0; q < 1 + ADJ_MAXA; ++q) r.d[q] = a.d[q] + b.d[q]; break;
        case OP_SUB: r.v = a.v - b.v; for (int q = 0; q < 1 + ADJ_MAXA; ++q) r.d[q] = a.d[q] - b.d[q]; break;
        case OP_MUL: r.v = a.v * b.v; for (int q = 0; q < 1 + ADJ_MAXA; ++q) r.d[q] = a.d[q] * b.v + a.v * b.d[q]; break;
        case OP_DIV: {
            r.v = a.v / b.v;
            for (int q = 0; q < 1 + ADJ_MAXA; ++q) r.d[q] = (a.d[q] - r.v * b.d[q]) / b.v;
            break;
        }
        case OP_MAX: r = (a.v >= b.v || b.v != b.v) ? a : b; break;  // fmax: NaN-ignoring, ties keep a
        case OP_MIN: r = (a.v <= b.v || b.v != b.v) ? a : b; break;
        default: r.v = Real(0); break;
        }
        st[sp - 1] = r;
    }
    return st[0];
}

// keys: the launch's Philox round keys when every contract has one seed.
template <class Real>
__device__ __forceinline__ void draws4(const AdjArgs &A, const PhiloxKeys &keys, uint64_t path, uint64_t d,
                                       Real z[4]) {
    if (A.z64 == nullptr && A.z32 == nullptr) {
        const uint4 ctr = make_uint4((uint32_t)(d >> 2), (uint32_t)path, (uint32_t)(path >> 32), 0u);
        const uint4 w = keys.ok ? philox4x32_10_rk(ctr, keys.rk)
                                : philox4x32_10(ctr, (uint32_t)A.seed, (uint32_t)(A.seed >> 32));
        box_muller(w.x, w.y, z[0], z[1]);
        box_muller(w.z, w.w, z[2], z[3]);
    } else {
        for (int j = 0; j < 4; ++j) {
            const uint64_t q = d + j;
            z[j] = q < A.z_dpp ? (A.z64 ? (Real)A.z64[path * A.z_dpp + q] : (Real)A.z32[path * A.z_dpp + q]) : Real(0);
        }
    }
}

// A contract's parameters in the path precision, converted once per path:
// GB300's FP64 pipe is a small fraction of its FP32 one, so no double is
// converted inside the step loops.
template <class Real>
struct AdjPar {
    Real mu, sigma, drift, r, kappa, theta, sigma_v, rho, rho_perp, drp, inv_w, s0;
    Real thr[ADJ_MAXU];
    // the barrier test of smoothed until u as sgn[u] * y >= hit[u] (strict
    // comparisons made inclusive at the next representable threshold)
    Real sgn[ADJ_MAXU], hit[ADJ_MAXU];
};

template <class Real>
__device__ __forceinline__ AdjPar<Real> adj_par(const AdjArgs &A) {
    AdjPar<Real> p;
    p.mu = (Real)A.mu;
    p.sigma = (Real)A.sigma;
    p.drift = sub_rn(p.mu, mul_rn(mul_rn(Real(0.5), p.sigma), p.sigma));
    p.r = (Real)A.r;
    p.kappa = (Real)A.kappa;
    p.theta = (Real)A.theta;
    p.sigma_v = (Real)A.sigma_v;
    p.rho = (Real)A.rho;
    p.rho_perp = (Real)A.rho_perp;
    p.drp = A.rho_perp > 0 ? (Real)(-A.rho / A.rho_perp) : Real(0);
    p.inv_w = (Real)A.inv_w;
    p.s0 = (Real)A.s0;
    for (int u = 0; u < ADJ_MAXU; ++u) {
        const Real t = u < A.n_su ? (Real)A.su[u].thr : Real(0);
        const int cmp = u < A.n_su ? A.su[u].cmp : CMP_GE;
        p.thr[u] = t;
        const bool down = cmp == CMP_LE || cmp == CMP_LT;
        p.sgn[u] = down ? Real(-1) : Real(1);
        // y > t  <=>  y >= next_up(t);  y < t  <=>  -y >= -next_down(t)
        const Real ti = cmp == CMP_GT ? next_up(t) : cmp == CMP_LT ? next_down(t) : t;
        p.hit[u] = down ? -ti : ti;
    }
    return p;
}

// One model step k (from k-1), returning the new (y, v) and the draws used.
template <class Real, int MODEL>
__device__ __forceinline__ void model_step(const AdjPar<Real> &p, int scheme, const StepRec<Real> &rec, Real z1,
                                           Real z2, Real &y, Real &v) {
    if (MODEL == KX_MODEL_GBM) {
        y = gbm_step(y, mul_rn(p.drift, rec.c0), mul_rn(p.sigma, rec.c1), z1);
    } else {
        heston_step<Real>(p.r, p.kappa, p.theta, p.sigma_v, p.rho, p.rho_perp, scheme, rec.c0, rec.c1, z1, z2, y, v);
    }
}

// One launch covers a list of contracts (each with its own model, grid and
// path count): the global path index runs over all of them (prefix offsets
// `off`), so an uneven book is one persistent launch.
//
// ACC: some contract keeps averages or running extrema. Without them the
// per-step work is the model step, the smoothed barriers and, only at the
// steps that pay flows (sorted by step on the host), the amounts.
template <class Real, int MODEL, bool ACC>
__global__ void __launch_bounds__(ADJ_BLOCK) k_adjoint(const AdjArgs *__restrict__ all, const uint64_t *__restrict__ off,
                                                       int n_contracts, uint64_t total, double *__restrict__ out,
                                                       const PhiloxKeys keys) {
    constexpr int DRAWS = MODEL == KX_MODEL_GBM ? 1 : 2;
    for (uint64_t gp = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; gp < total;
         gp += (uint64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_contracts - 1;  // contract of global path gp
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= gp) lo = mid;
            else hi = mid - 1;
        }
        const AdjArgs &A = all[lo];
        const uint64_t path = gp - off[lo];
        const StepRec<Real> *R = reinterpret_cast<const StepRec<Real> *>(A.steps);
        const KxProgram &P = *A.P;
        const int N = A.n_times - 1;  // steps
        const int K = A.K;
        const AdjPar<Real> pp = adj_par<Real>(A);
        const Real s0 = pp.s0;
        const Real inv_w = pp.inv_w;
        // ------------------------------ forward ------------------------------
        Real ck_y[ADJ_MAXCK], ck_v[ADJ_MAXCK];
        Real y = Real(0), v = (Real)fmax(A.v0, 0.0);
        Real accv[ADJ_MAXA], accraw[ADJ_MAXA];
        int argx[ADJ_MAXA];
        for (int a = 0; a < ADJ_MAXA; ++a) {
            accraw[a] = a < A.n_acc ? (A.acc[a].kind == ACC_MAX ? Real(-INFINITY) : A.acc[a].kind == ACC_MIN ? Real(INFINITY) : Real(0)) : Real(0);
            argx[a] = 0;
            accv[a] = Real(0);
        }
        Real surv[ADJ_MAXU];
        int knock[ADJ_MAXU];  // first step the (unsmoothed) barrier holds
        for (int u = 0; u < ADJ_MAXU; ++u) {
            surv[u] = Real(1);
            knock[u] = INT_MAX;
        }
        double pv_hard = 0.0;
        // flow records
        double fP[ADJ_MAXF];
        Real fcs[ADJ_MAXF], fca[ADJ_MAXF][ADJ_MAXA];
        int farg[ADJ_MAXF][ADJ_MAXA];
        double pv = 0.0, pv_t = 0.0;  // price and sum_f t_f P_f
        const int nflows = A.n_flows;
        const int nsu = A.n_su;
        int su_arm[ADJ_MAXU];
        for (int u = 0; u < ADJ_MAXU; ++u) su_arm[u] = u < nsu ? A.su[u].arm : INT_MAX;
        int ck = 0, next_ck = 0;                          // next checkpoint slot and its step
        int nf = 0;                                       // next flow (flows sorted by step)
        int nft = nflows > 0 ? A.flow[0].t : INT_MAX;     // its step
        Real z[4];
        for (int k = 0; k <= N; ++k) {
            if (k > 0) {
                const uint64_t d = (uint64_t)(k - 1) * DRAWS;
                if ((d & 3u) == 0) draws4<Real>(A, keys, path, d, z);
                const int q = (int)(d & 3u);
                model_step<Real, MODEL>(pp, A.scheme, R[k], z[q], DRAWS == 2 ? z[q + 1] : Real(0), y, v);
            }
            if (k == next_ck) {  // checkpoint every K steps
                ck_y[ck] = y;
                ck_v[ck] = v;
                ++ck;
                next_ck += K;
            }
            const bool pays = k == nft;
            // the spot and the sums rounded once each (no contraction into FMAs), so that
            // k_adjoint_gbm_acc, which repeats these operations, gives the same values
            const Real S = (ACC || pays) ? spot_of<Real>(s0, y) : Real(0);
            if (ACC)
                for (int a = 0; a < A.n_acc; ++a) {
                    const AdjAcc &Ac = A.acc[a];
                    if (k < Ac.i_from || k > Ac.i_to) continue;
                    if (Ac.kind == ACC_MAX) { if (S > accraw[a]) { accraw[a] = S; argx[a] = k; } }
                    else if (Ac.kind == ACC_MIN) { if (S < accraw[a]) { accraw[a] = S; argx[a] = k; } }
                    else accraw[a] = add_rn(accraw[a], S);
                }
            for (int u = 0; u < nsu; ++u)
                if (k >= su_arm[u]) {
                    const Real x = pp.sgn[u] * (y - pp.thr[u]) * inv_w;  // > 0 beyond the barrier
                    if (x > smooth_cut<Real>()) surv[u] *= logistic(x);  // weight 1 below the cut
                    const bool hit = pp.sgn[u] * y >= pp.hit[u];
                    if (hit && knock[u] == INT_MAX) knock[u] = k;
                }
            if (!pays) continue;
            for (int f = nf; f < nflows && A.flow[f].t == k; ++f) {
                const AdjFlow &F = A.flow[f];
                nf = f + 1;
                if (ACC)
                    for (int a = 0; a < A.n_acc; ++a)
                    accv[a] = A.acc[a].kind == ACC_SUM ? accraw[a] / (Real)(min(k, A.acc[a].i_to) - A.acc[a].i_from + 1)
                                                       : accraw[a];
                Dual<Real> amt;
                if (F.kind == AK_CONST) {
                    amt.v = (Real)F.sign;
                    for (int q = 0; q < 1 + ADJ_MAXA; ++q) amt.d[q] = Real(0);
                } else {
                    amt = eval_dual<Real>(P, F.code_off, F.code_len, S, accv);
                }
                Real w = Real(1);
                for (int u = 0; u < A.n_su; ++u)
                    if ((F.su_mask >> u) & 1u) w *= surv[u];
                const double df = A.disc[k];
                fP[f] = (double)amt.v * (double)w * df;
                fcs[f] = (Real)((double)(amt.d[0] * w) * df);
                for (int a = 0; a < ADJ_MAXA; ++a) {
                    Real c = (Real)((double)(amt.d[1 + a] * w) * df);
                    if (a < A.n_acc && A.acc[a].kind == ACC_SUM)
                        c /= (Real)(min(k, A.acc[a].i_to) - A.acc[a].i_from + 1);
                    fca[f][a] = c;
                    farg[f][a] = argx[a];
                }
                pv += fP[f];
                pv_t += A.times[k] * fP[f];
                bool alive = true;  // the flow under the hard barriers (pricer.rs:407-413)
                for (int u = 0; u < A.n_su; ++u)
                    if (((F.su_mask >> u) & 1u) && knock[u] <= k) alive = false;
                if (alive) pv_hard += (double)amt.v * df;
            }
            nft = nf < nflows ? A.flow[nf].t : INT_MAX;
        }
        // ------------------------------ reverse ------------------------------
        Real sy[ADJ_KMAX + 1], sv[ADJ_KMAX + 1], sz1[ADJ_KMAX + 1], sz2[ADJ_KMAX + 1];
        Real lam = Real(0), mu = Real(0);  // dPV/dy_{k+1}, dPV/dv_{k+1}
        Real Q[ADJ_MAXU] = {};             // sum of P_f (t_f >= k) under each smoothed until
        Real G[ADJ_MAXA] = {};             // per average: sum of coefficients whose window holds k
        Real g_sig = 0, g_r = 0, g_k = 0, g_th = 0, g_sv = 0, g_rho = 0;
        int pf = nflows - 1;                              // last flow not yet swept
        int pft = pf >= 0 ? A.flow[pf].t : -1;            // its step
        const int nseg = (N + K - 1) / K;
        for (int c = nseg - 1; c >= 0; --c) {
            const int k0 = c * K;
            const int k1 = min(k0 + K, N);
            // recompute states k0..k1 and the draws of steps k0+1..k1
            Real yy = ck_y[c], vv = ck_v[c];
            sy[0] = yy;
            sv[0] = vv;
            for (int k = k0 + 1; k <= k1; ++k) {
                const uint64_t d = (uint64_t)(k - 1) * DRAWS;
                if ((d & 3u) == 0 || k == k0 + 1) draws4<Real>(A, keys, path, d & ~3ull, z);
                const int q = (int)(d & 3u);
                const Real a1 = z[q], a2 = DRAWS == 2 ? z[q + 1] : Real(0);
                model_step<Real, MODEL>(pp, A.scheme, R[k], a1, a2, yy, vv);
                sy[k - k0] = yy;
                sv[k - k0] = vv;
                sz1[k - k0] = a1;
                sz2[k - k0] = a2;
            }
            const int ktop = (c == nseg - 1) ? k1 : k1 - 1;
            for (int k = ktop; k >= k0; --k) {
                const int j = k - k0;
                if (k < N) {
                    // adjoint of step k -> k+1 (state k, draws of step k+1)
                    const StepRec<Real> rec = R[k + 1];
                    const Real dt = rec.c0, sq = rec.c1;
                    const Real z1 = sz1[j + 1], z2 = sz2[j + 1];
                    if (MODEL == KX_MODEL_GBM) {
                        g_sig += lam * (-pp.sigma * dt + sq * z1);
                        g_r += lam * dt;
                    } else {
                        const Real vk = sv[j];
                        const bool ft = A.scheme == KX_HESTON_FULL_TRUNCATION;
                        const Real vp = ft ? fmax(vk, Real(0)) : vk;
                        const Real dvp = (ft && vk <= Real(0)) ? Real(0) : Real(1);
                        const Real sqv = sqrt(vp);
                        const Real dsq = sqv > Real(0) ? Real(0.5) / sqv : Real(0);  // d sqrt(v)/dv, 0 at v = 0
                        const Real mix = pp.rho * z1 + pp.rho_perp * z2;
                        // v_{k+1} before the floor; the floor passes the adjoint only where it did not bite
                        const Real vn = vk + pp.kappa * (pp.theta - vp) * dt + pp.sigma_v * sqv * mix * sq;
                        const Real m = (ft || vn > Real(0)) ? mu : Real(0);
                        const Real dx_dv = (Real(-0.5) * dt + z1 * sq * dsq) * dvp;
                        const Real dvn_dv = Real(1) + (-pp.kappa * dt + pp.sigma_v * mix * sq * dsq) * dvp;
                        g_r += lam * dt;
                        g_k += m * (pp.theta - vp) * dt;
                        g_th += m * pp.kappa * dt;
                        g_sv += m * sqv * mix * sq;
                        g_rho += m * pp.sigma_v * sqv * (z1 + pp.drp * z2) * sq;
                        mu = lam * dx_dv + m * dvn_dv;
                    }
                }
                // direct contributions at state k
                const Real yk = sy[j];
                Real g = Real(0);
                if (ACC) {
                    const Real Sk = spot_of<Real>(s0, yk);
                    for (int f = 0; f < nflows; ++f) {
                        // an average read at t_f covers [i_from, min(t_f, i_to)]: its coefficient
                        // joins when the sweep reaches the window's last step
                        for (int a = 0; a < A.n_acc; ++a)
                            if (A.acc[a].kind == ACC_SUM && k == min(A.flow[f].t, A.acc[a].i_to)) G[a] += fca[f][a];
                        if (A.flow[f].t != k) continue;
                        g += fcs[f] * Sk;
                        for (int u = 0; u < A.n_su; ++u)
                            if ((A.flow[f].su_mask >> u) & 1u) Q[u] += (Real)fP[f];
                    }
                    for (int f = 0; f < nflows; ++f)  // running max/min: at the arg-extremum
                        if (A.flow[f].t >= k)
                            for (int a = 0; a < A.n_acc; ++a)
                                if (A.acc[a].kind != ACC_SUM && farg[f][a] == k) g += fca[f][a] * Sk;
                    for (int a = 0; a < A.n_acc; ++a)  // averages: inside the window
                        if (A.acc[a].kind == ACC_SUM && k >= A.acc[a].i_from) g += G[a] * Sk;
                } else if (k == pft) {  // the flows paid at step k, in slot order
                    const Real Sk = spot_of<Real>(s0, yk);
                    int f0 = pf;
                    while (f0 > 0 && A.flow[f0 - 1].t == k) --f0;
                    for (int f = f0; f <= pf; ++f) {
                        g += fcs[f] * Sk;
                        for (int u = 0; u < A.n_su; ++u)
                            if ((A.flow[f].su_mask >> u) & 1u) Q[u] += (Real)fP[f];
                    }
                    pf = f0 - 1;
                    pft = pf >= 0 ? A.flow[pf].t : -1;
                }
                for (int u = 0; u < nsu; ++u)
                    if (k >= su_arm[u] && Q[u] != Real(0)) {
                        const Real x = pp.sgn[u] * (yk - pp.thr[u]) * inv_w;
                        if (x > smooth_cut<Real>()) {  // below the cut the weight is 1: no term
                            const Real s = logistic(x);
                            const Real dls = (Real(1) - s) * inv_w;  // |d log s / dy|
                            g -= Q[u] * pp.sgn[u] * dls;
                        }
                    }
                // leaving an average window when walking below its first step
                if (ACC)
                    for (int a = 0; a < A.n_acc; ++a)
                        if (A.acc[a].kind == ACC_SUM && k == A.acc[a].i_from) G[a] = Real(0);
                lam += g;
            }
        }
        double *o = out + A.out_off + path;
        const uint64_t n = total;
        o[8 * n] = pv_hard;
        o[0 * n] = pv;
        o[1 * n] = (double)lam / A.s0;                  // d/ds0
        if (MODEL == KX_MODEL_GBM) {
            o[2 * n] = (double)g_sig;                    // d/dsigma
            o[3 * n] = (double)g_r - pv_t;               // d/dr: drift and discount
        } else {
            o[2 * n] = A.v0 > 0 ? (double)mu : 0.0;      // d/dv0
            o[3 * n] = (double)g_r - pv_t;               // d/dr
            o[4 * n] = (double)g_k;                      // d/dkappa
            o[5 * n] = (double)g_th;                     // d/dtheta
            o[6 * n] = (double)g_sv;                     // d/dsigma_v
            o[7 * n] = (double)g_rho;                    // d/drho
        }
    }
}

// Static schedule of a supported contract on a grid (host).
static void schedule(const Lowered &low, const KxProgram &P, const StepTables &tab, const Model &m, AdjArgs &a) {
    const int n = P.n_times;
    const int NEVER = INT_MAX;
    // the slot whose firing arms slot i (-1: armed at step 0)
    std::vector<int> parent(P.n_trig, -1);
    for (int i = 0; i < P.n_trig; ++i)
        for (int j = 0; j < P.n_trig; ++j)
            if ((P.trig[i].fire_arm >> j) & 1u) parent[j] = i;
    std::vector<int> arm(P.n_trig, NEVER), fire(P.n_trig, NEVER);
    auto first_from = [&](int i, int from) {
        for (int k = std::max(from, 0); k < n; ++k)
            if ((tab.time_true[k] >> i) & 1u) return k;
        return NEVER;
    };
    for (int i = 0; i < P.n_trig; ++i) {  // slots are numbered parents first
        const KxTrig &T = P.trig[i];
        arm[i] = parent[i] < 0 ? 0 : fire[parent[i]];
        if (T.kind == TK_WHEN) {
            if (T.cond_kind != CK_TIME)
                raise(KX_UNSUPPORTED, "adjoint: when/anytime conditions must depend on time only");
            fire[i] = arm[i] == NEVER ? NEVER : first_from(i, arm[i]);
        } else {
            if (T.cond_kind == CK_TIME) fire[i] = arm[i] == NEVER ? NEVER : first_from(i, arm[i]);  // knock step
            else if (T.cond_kind != CK_SPOT_CMP)
                raise(KX_UNSUPPORTED, "adjoint: until conditions must be Spot vs Const or time only");
        }
    }
    for (int a2 = 0; a2 < P.n_acc; ++a2)
        if (P.acc[a2].inner != IK_SPOT) raise(KX_UNSUPPORTED, "adjoint: averages / running extrema must be of the spot");
    if (P.n_acc > ADJ_MAXA) raise(KX_UNSUPPORTED, "adjoint: at most 2 averages / running extrema");
    a.n_acc = P.n_acc;
    for (int q = 0; q < P.n_acc; ++q) {
        a.acc[q].kind = P.acc[q].kind;
        a.acc[q].i_from = P.acc[q].i_from;
        a.acc[q].i_to = P.acc[q].i_to;
        if (P.acc[q].kind == ACC_SUM && P.acc[q].static_err) raise(KX_MALFORMED_CONTRACT, "empty average window");
    }
    // smoothed untils
    std::vector<int> su_index(P.n_trig, -1);
    a.n_su = 0;
    for (int i = 0; i < P.n_trig; ++i) {
        const KxTrig &T = P.trig[i];
        if (T.kind != TK_UNTIL || T.cond_kind != CK_SPOT_CMP || arm[i] == NEVER) continue;
        if (a.n_su >= ADJ_MAXU) raise(KX_UNSUPPORTED, "adjoint: at most 2 barrier untils");
        su_index[i] = a.n_su;
        AdjUntil &U = a.su[a.n_su++];
        U.arm = arm[i];
        U.cmp = T.cmp;
        U.thr = std::log(low.spot_cmp[T.spot_slot].c / m.s0);
    }
    // live flows
    a.n_flows = 0;
    for (int j = 0; j < P.n_leaf; ++j) {
        int acq = -1;
        for (int i = 0; i < P.n_trig; ++i)
            if (P.trig[i].kind == TK_WHEN && ((P.trig[i].leaves >> j) & 1u)) acq = i;
        const int t = acq < 0 ? 0 : fire[acq];
        if (t == NEVER) continue;
        bool dead = false;
        uint32_t mask = 0;
        for (int i = 0; i < P.n_trig; ++i) {
            const KxTrig &T = P.trig[i];
            if (T.kind != TK_UNTIL || !((T.leaves >> j) & 1u)) continue;
            if (T.cond_kind == CK_TIME && fire[i] <= t) dead = true;  // knocked at or before the flow
            if (su_index[i] >= 0) mask |= 1u << su_index[i];
        }
        if (dead) continue;
        if (a.n_flows >= ADJ_MAXF) raise(KX_UNSUPPORTED, "adjoint: at most 4 flows");
        const KxLeaf &F = P.leaf[j];
        for (int c = F.code_off; c < F.code_off + F.code_len; ++c) {
            const uint8_t op = P.code[c].op;
            if (op == OP_ACC && P.acc[P.code[c].arg].kind == ACC_SUM) {
                const KxAcc &Ac = P.acc[P.code[c].arg];
                if (Ac.fixed && Ac.i_to > t) raise(KX_UNSUPPORTED, "adjoint: average window ends after the flow date");
                if (!Ac.fixed && t < Ac.e_min) raise(KX_MALFORMED_CONTRACT, "average window inverted at the flow date");
            }
        }
        AdjFlow &fl = a.flow[a.n_flows++];
        fl.t = t;
        fl.kind = F.kind;
        fl.code_off = F.code_off;
        fl.code_len = F.code_len;
        fl.sign = F.sign;
        fl.su_mask = mask;
    }
    // by payment step (slot order within a step): the kernels walk them in order
    std::stable_sort(a.flow, a.flow + a.n_flows, [](const AdjFlow &x, const AdjFlow &y) { return x.t < y.t; });
}

// GBM contracts without averages or running extrema, checkpoint interval K
// fixed at compile time: the recomputed segment (K + 1 states and K draws)
// lives in registers, the segment loops are unrolled, and the GBM step's
// Jacobian (d y_{k+1} / d y_k = 1) leaves the adjoint unchanged across a
// step. Same quantities as k_adjoint.
//
// The checkpoints and the per-flow records of a path live in shared memory,
// one column per thread (ck[c * ADJ_BLOCK + t], the flows' values after the
// checkpoints), so that registers hold only the state of the step loops and
// eight blocks (FP32; four in FP64) fit an SM: n_ck checkpoint rows are
// allocated at launch.
template <class Real, int K, int NSU, int MINB>
__global__ void __launch_bounds__(ADJ_BLOCK, MINB) k_adjoint_gbm(const AdjArgs *__restrict__ all,
                                                              const uint64_t *__restrict__ off, int n_contracts,
                                                              uint64_t total, double *__restrict__ out,
                                                              const PhiloxKeys keys, int n_ck) {
    static_assert(K % 4 == 0 && (K & (K - 1)) == 0 && K <= ADJ_KMAX, "K: a power of two, multiple of 4");
    extern __shared__ __align__(16) unsigned char adj_smem[];
    double *const fP = reinterpret_cast<double *>(adj_smem) + threadIdx.x;                  // [ADJ_MAXF][ADJ_BLOCK]
    Real *const fcs = reinterpret_cast<Real *>(adj_smem + ADJ_MAXF * ADJ_BLOCK * sizeof(double)) + threadIdx.x;
    Real *const ck_y = fcs + ADJ_MAXF * ADJ_BLOCK;                                          // [n_ck][ADJ_BLOCK]
    for (uint64_t gp = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; gp < total;
         gp += (uint64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_contracts - 1;  // contract of global path gp
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= gp) lo = mid;
            else hi = mid - 1;
        }
        const AdjArgs &A = all[lo];
        const uint64_t path = gp - off[lo];
        const StepRec<Real> *R = reinterpret_cast<const StepRec<Real> *>(A.steps);
        const KxProgram &P = *A.P;
        const int N = A.n_times - 1;
        const AdjPar<Real> pp = adj_par<Real>(A);
        const Real s0 = pp.s0, inv_w = pp.inv_w;
        const int nflows = A.n_flows;
        constexpr int nsu = NSU;
        const bool uni = A.uniform != 0;
        const Real udt = (Real)A.uc0, usq = (Real)A.uc1;
        const Real ua = mul_rn(pp.drift, udt), ub = mul_rn(pp.sigma, usq);  // uniform grids: the step's terms
        int su_arm[ADJ_MAXU];
#pragma unroll
        for (int u = 0; u < ADJ_MAXU; ++u) su_arm[u] = u < nsu ? A.su[u].arm : INT_MAX;
        // ------------------------------ forward ------------------------------
        Real y = Real(0);
        Real surv[ADJ_MAXU];
        int knock[ADJ_MAXU];
        for (int u = 0; u < ADJ_MAXU; ++u) {
            surv[u] = Real(1);
            knock[u] = INT_MAX;
        }
        double pv_hard = 0.0, pv = 0.0, pv_t = 0.0;
        int nf = 0, nft = nflows > 0 ? A.flow[0].t : INT_MAX;
        Real z0 = 0, z1 = 0, z2 = 0, z3 = 0;
        for (int k = 0; k <= N; ++k) {
            if (k > 0) {
                const int q = (k - 1) & 3;
                if (q == 0) {
                    Real z[4];
                    draws4<Real>(A, keys, path, (uint64_t)(k - 1), z);
                    z0 = z[0]; z1 = z[1]; z2 = z[2]; z3 = z[3];
                }
                const Real zk = q == 0 ? z0 : q == 1 ? z1 : q == 2 ? z2 : z3;
                y = uni ? gbm_step(y, ua, ub, zk)
                        : gbm_step(y, mul_rn(pp.drift, R[k].c0), mul_rn(pp.sigma, R[k].c1), zk);
            }
            if (k % K == 0) ck_y[(k / K) * ADJ_BLOCK] = y;  // K is a power of two: a mask, not a division
#pragma unroll
            for (int u = 0; u < nsu; ++u)
                if (k >= su_arm[u]) {
                    const Real x = pp.sgn[u] * (y - pp.thr[u]) * inv_w;
                    if (x > smooth_cut<Real>()) surv[u] *= logistic(x);  // weight 1 below the cut
                    if (pp.sgn[u] * y >= pp.hit[u] && knock[u] == INT_MAX) knock[u] = k;
                }
            if (k != nft) continue;
            const Real S = spot_of<Real>(s0, y);
            for (int f = nf; f < nflows && A.flow[f].t == k; ++f) {
                const AdjFlow &F = A.flow[f];
                nf = f + 1;
                Dual<Real> amt;
                if (F.kind == AK_CONST) {
                    amt.v = (Real)F.sign;
                    for (int q = 0; q < 1 + ADJ_MAXA; ++q) amt.d[q] = Real(0);
                } else {
                    Real none[ADJ_MAXA] = {};
                    amt = eval_dual<Real>(P, F.code_off, F.code_len, S, none);
                }
                Real w = Real(1);
#pragma unroll
                for (int u = 0; u < nsu; ++u)
                    if ((F.su_mask >> u) & 1u) w *= surv[u];
                const double df = A.disc[k];
                const double fpv = (double)amt.v * (double)w * df;
                fP[f * ADJ_BLOCK] = fpv;
                fcs[f * ADJ_BLOCK] = (Real)((double)(amt.d[0] * w) * df);
                pv += fpv;
                pv_t += A.times[k] * fpv;
                bool alive = true;
#pragma unroll
                for (int u = 0; u < nsu; ++u)
                    if (((F.su_mask >> u) & 1u) && knock[u] <= k) alive = false;
                if (alive) pv_hard += (double)amt.v * df;
            }
            nft = nf < nflows ? A.flow[nf].t : INT_MAX;
        }
        // ------------------------------ reverse ------------------------------
        Real lam = Real(0);  // dPV/dy_{k+1}
        Real Q[ADJ_MAXU] = {};
        Real g_sig = Real(0), g_r = Real(0);
        int pf = nflows - 1, pft = pf >= 0 ? A.flow[pf].t : -1;
        const int nseg = (N + K - 1) / K;
        for (int c = nseg - 1; c >= 0; --c) {
            const int k0 = c * K;
            const int k1 = min(k0 + K, N);
            Real sy[K + 1], sz[K + 2];
            sy[0] = ck_y[c * ADJ_BLOCK];
            sz[K + 1] = Real(0);
#pragma unroll
            for (int q = 0; q < K / 4; ++q) {  // the draws of steps k0 + 1 .. k0 + K
                Real w4[4];
                draws4<Real>(A, keys, path, (uint64_t)(k0 + 4 * q), w4);
#pragma unroll
                for (int j = 0; j < 4; ++j) sz[1 + 4 * q + j] = w4[j];
            }
            if (uni) {  // one branch per segment, none per step
#pragma unroll
                for (int j = 1; j <= K; ++j) sy[j] = gbm_step(sy[j - 1], ua, ub, sz[j]);
            } else {
#pragma unroll
                for (int j = 1; j <= K; ++j) {
                    const StepRec<Real> rec = R[min(k0 + j, N)];  // past N: harmless states never read
                    sy[j] = gbm_step(sy[j - 1], mul_rn(pp.drift, rec.c0), mul_rn(pp.sigma, rec.c1), sz[j]);
                }
            }
            const int jtop = (c == nseg - 1) ? k1 - k0 : k1 - k0 - 1;
#pragma unroll
            for (int j = K; j >= 0; --j) {
                if (j > jtop) continue;
                const int k = k0 + j;
                if (k < N) {  // step k -> k + 1: d y_{k+1} / d y_k = 1, so lam carries over
                    Real dt = udt, sq = usq;
                    if (!uni) {
                        const StepRec<Real> rn = R[k + 1];
                        dt = rn.c0;
                        sq = rn.c1;
                    }
                    g_sig += lam * (-pp.sigma * dt + sq * sz[j + 1]);
                    g_r += lam * dt;
                }
                const Real yk = sy[j];
                Real g = Real(0);
                if (k == pft) {  // the flows paid at step k, in slot order
                    const Real Sk = spot_of<Real>(s0, yk);
                    int f0 = pf;
                    while (f0 > 0 && A.flow[f0 - 1].t == k) --f0;
                    for (int f = f0; f <= pf; ++f) {
                        g += fcs[f * ADJ_BLOCK] * Sk;
#pragma unroll
                        for (int u = 0; u < nsu; ++u)
                            if ((A.flow[f].su_mask >> u) & 1u) Q[u] += (Real)fP[f * ADJ_BLOCK];
                    }
                    pf = f0 - 1;
                    pft = pf >= 0 ? A.flow[pf].t : -1;
                }
#pragma unroll
                for (int u = 0; u < nsu; ++u)
                    if (k >= su_arm[u] && Q[u] != Real(0)) {
                        const Real x = pp.sgn[u] * (yk - pp.thr[u]) * inv_w;
                        if (x > smooth_cut<Real>()) {  // below the cut the weight is 1: no term
                            const Real sv = logistic(x);
                            const Real dls = (Real(1) - sv) * inv_w;
                            g -= Q[u] * pp.sgn[u] * dls;
                        }
                    }
                lam += g;
            }
        }
        double *o = out + A.out_off + path;
        const uint64_t n = total;
        o[8 * n] = pv_hard;
        o[0 * n] = pv;
        o[1 * n] = (double)lam / A.s0;
        o[2 * n] = (double)g_sig;
        o[3 * n] = (double)g_r - pv_t;
    }
}

// Per-thread records of the GBM adjoint kernels in shared memory, one column
// per thread (entry e of thread t at e * ADJ_BLOCK + t), sized per launch:
// nf flow values (double), nf spot coefficients, nf * na accumulator
// coefficients and arg-extremum steps, n_ck checkpoints, and the K + 1
// states and normals of the segment being swept.
struct AdjSmem {
    int nf, na, n_ck, K;
};
template <class Real>
__host__ __device__ inline size_t adj_smem_bytes(const AdjSmem &L) {
    return (size_t)ADJ_BLOCK * (L.nf * sizeof(double) +
                                (L.nf + L.nf * L.na + L.n_ck + 2 * (L.K + 1)) * sizeof(Real) + L.nf * L.na * sizeof(int));
}

// GBM contracts with averages or running extrema (Asians, lookbacks, their
// barrier versions) and, with none, barrier and European contracts: the
// checkpoint interval K is a launch parameter, the accumulators live in
// registers, everything indexed by step in shared memory (AdjSmem), so the
// step loops are short and not unrolled. Every quantity is computed with
// k_adjoint's operations in k_adjoint's order, so the two kernels give the
// same outputs; what changes is the bookkeeping:
//  * on a uniform grid the step coefficients are formed once per path (the
//    products k_adjoint forms at every step, same roundings);
//  * the reverse sweep knows the next step at which something other than the
//    step-by-step terms happens (a flow paid, an average's coefficient joining
//    at min(t_f, window end), a running extremum's arg-extremum) and tests
//    one step number per step.
// NAC, AK0, NS: the launch's accumulator count, the kind of its first
// accumulator and its smoothed-barrier count when every contract of the
// launch shares them (-1: read per contract), so that the checks they decide
// leave the step loops.
template <class Real, int MINB, int NAC = -1, int AK0 = -1, int NS = -1>
__global__ void __launch_bounds__(ADJ_BLOCK, MINB)
    k_adjoint_gbm_acc(const AdjArgs *__restrict__ all, const uint64_t *__restrict__ off, int n_contracts,
                      uint64_t total, double *__restrict__ out, const PhiloxKeys keys, const AdjSmem L) {
    extern __shared__ __align__(16) unsigned char adj_smem[];
    constexpr int B = ADJ_BLOCK;
    const int K = L.K, NA = L.na;
    double *const fP = reinterpret_cast<double *>(adj_smem) + threadIdx.x;                    // [f]
    Real *const fcs = reinterpret_cast<Real *>(adj_smem + (size_t)B * L.nf * sizeof(double)) + threadIdx.x;  // [f]
    Real *const fca = fcs + (size_t)B * L.nf;                                                 // [f * NA + a]
    Real *const ck_y = fca + (size_t)B * L.nf * NA;                                           // [c]
    Real *const sy = ck_y + (size_t)B * L.n_ck;                                               // [j], j <= K
    Real *const sz = sy + (size_t)B * (K + 1);                                                // [j - 1], 1 <= j <= K
    int *const farg = reinterpret_cast<int *>(sz + (size_t)B * (K + 1) - threadIdx.x) + threadIdx.x;  // [f * NA + a]
    for (uint64_t gp = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; gp < total;
         gp += (uint64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_contracts - 1;  // contract of global path gp
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= gp) lo = mid;
            else hi = mid - 1;
        }
        const AdjArgs &A = all[lo];
        const uint64_t path = gp - off[lo];
        const StepRec<Real> *R = reinterpret_cast<const StepRec<Real> *>(A.steps);
        const KxProgram &P = *A.P;
        const int N = A.n_times - 1;
        const AdjPar<Real> pp = adj_par<Real>(A);
        const Real s0 = pp.s0, inv_w = pp.inv_w;
        const int nflows = A.n_flows;
        const int nsu = NS >= 0 ? NS : A.n_su, nacc = NAC >= 0 ? NAC : A.n_acc;
        const bool uni = A.uniform != 0;
        const Real udt = (Real)A.uc0, usq = (Real)A.uc1;
        const Real ua = mul_rn(pp.drift, udt), ub = mul_rn(pp.sigma, usq);  // uniform grids: the step's terms
        int su_arm[ADJ_MAXU], a_kind[ADJ_MAXA], a_from[ADJ_MAXA], a_to[ADJ_MAXA];
#pragma unroll
        for (int u = 0; u < ADJ_MAXU; ++u) su_arm[u] = u < nsu ? A.su[u].arm : INT_MAX;
#pragma unroll
        for (int a = 0; a < ADJ_MAXA; ++a) {
            a_kind[a] = a == 0 && AK0 >= 0 ? AK0 : a < nacc ? A.acc[a].kind : ACC_SUM;
            a_from[a] = a < nacc ? A.acc[a].i_from : INT_MAX;
            a_to[a] = a < nacc ? A.acc[a].i_to : -1;
        }
        // ------------------------------ forward ------------------------------
        Real y = Real(0);
        Real accraw[ADJ_MAXA];
        int argx[ADJ_MAXA];
#pragma unroll
        for (int a = 0; a < ADJ_MAXA; ++a) {
            accraw[a] = a < nacc ? (a_kind[a] == ACC_MAX ? Real(-INFINITY) : a_kind[a] == ACC_MIN ? Real(INFINITY) : Real(0))
                                 : Real(0);
            argx[a] = 0;
        }
        Real surv[ADJ_MAXU];
        int knock[ADJ_MAXU];
#pragma unroll
        for (int u = 0; u < ADJ_MAXU; ++u) {
            surv[u] = Real(1);
            knock[u] = INT_MAX;
        }
        double pv_hard = 0.0, pv = 0.0, pv_t = 0.0;
        int nf = 0, nft = nflows > 0 ? A.flow[0].t : INT_MAX;
        Real z0 = 0, z1 = 0, z2 = 0, z3 = 0;
#pragma unroll 1
        for (int k = 0; k <= N; ++k) {
            if (k > 0) {
                const int q = (k - 1) & 3;
                if (q == 0) {
                    Real z[4];
                    draws4<Real>(A, keys, path, (uint64_t)(k - 1), z);
                    z0 = z[0]; z1 = z[1]; z2 = z[2]; z3 = z[3];
                }
                const Real zk = q == 0 ? z0 : q == 1 ? z1 : q == 2 ? z2 : z3;
                y = uni ? gbm_step(y, ua, ub, zk)
                        : gbm_step(y, mul_rn(pp.drift, R[k].c0), mul_rn(pp.sigma, R[k].c1), zk);
            }
            if (k % K == 0) ck_y[(k / K) * B] = y;
            const Real S = spot_of<Real>(s0, y);
#pragma unroll
            for (int a = 0; a < ADJ_MAXA; ++a) {
                if (a >= nacc || k < a_from[a] || k > a_to[a]) continue;
                if (a_kind[a] == ACC_MAX) { if (S > accraw[a]) { accraw[a] = S; argx[a] = k; } }
                else if (a_kind[a] == ACC_MIN) { if (S < accraw[a]) { accraw[a] = S; argx[a] = k; } }
                else accraw[a] = add_rn(accraw[a], S);
            }
#pragma unroll
            for (int u = 0; u < ADJ_MAXU; ++u)
                if (u < nsu && k >= su_arm[u]) {
                    const Real x = pp.sgn[u] * (y - pp.thr[u]) * inv_w;
                    if (x > smooth_cut<Real>()) surv[u] *= logistic(x);  // weight 1 below the cut
                    if (pp.sgn[u] * y >= pp.hit[u] && knock[u] == INT_MAX) knock[u] = k;
                }
            if (k != nft) continue;
            Real accv[ADJ_MAXA];
#pragma unroll
            for (int a = 0; a < ADJ_MAXA; ++a)
                accv[a] = a < nacc && a_kind[a] == ACC_SUM ? accraw[a] / (Real)(min(k, a_to[a]) - a_from[a] + 1)
                          : a < nacc ? accraw[a] : Real(0);
            for (int f = nf; f < nflows && A.flow[f].t == k; ++f) {
                const AdjFlow &F = A.flow[f];
                nf = f + 1;
                Dual<Real> amt;
                if (F.kind == AK_CONST) {
                    amt.v = (Real)F.sign;
                    for (int q = 0; q < 1 + ADJ_MAXA; ++q) amt.d[q] = Real(0);
                } else {
                    amt = eval_dual<Real>(P, F.code_off, F.code_len, S, accv);
                }
                Real w = Real(1);
#pragma unroll
                for (int u = 0; u < ADJ_MAXU; ++u)
                    if (u < nsu && ((F.su_mask >> u) & 1u)) w *= surv[u];
                const double df = A.disc[k];
                const double fpv = (double)amt.v * (double)w * df;
                fP[f * B] = fpv;
                fcs[f * B] = (Real)((double)(amt.d[0] * w) * df);
#pragma unroll
                for (int a = 0; a < ADJ_MAXA; ++a) {
                    if (a >= NA) continue;
                    Real c = (Real)((double)(amt.d[1 + a] * w) * df);
                    if (a < nacc && a_kind[a] == ACC_SUM) c /= (Real)(min(k, a_to[a]) - a_from[a] + 1);
                    fca[(f * NA + a) * B] = c;
                    farg[(f * NA + a) * B] = argx[a];
                }
                pv += fpv;
                pv_t += A.times[k] * fpv;
                bool alive = true;
#pragma unroll
                for (int u = 0; u < ADJ_MAXU; ++u)
                    if (u < nsu && ((F.su_mask >> u) & 1u) && knock[u] <= k) alive = false;
                if (alive) pv_hard += (double)amt.v * df;
            }
            nft = nf < nflows ? A.flow[nf].t : INT_MAX;
        }
        // ------------------------------ reverse ------------------------------
        // the next step (below lim) at which an average's coefficient joins, or
        // at which a running extremum of some flow was taken
        auto next_join = [&](int lim) {
            int m = -1;
            for (int f = 0; f < nflows; ++f)
#pragma unroll
                for (int a = 0; a < ADJ_MAXA; ++a)
                    if (a < nacc && a_kind[a] == ACC_SUM) {
                        const int s = min(A.flow[f].t, a_to[a]);
                        if (s < lim && s > m) m = s;
                    }
            return m;
        };
        auto next_ext = [&](int lim) {
            int m = -1;
            for (int f = 0; f < nflows; ++f)
#pragma unroll
                for (int a = 0; a < ADJ_MAXA; ++a)
                    if (a < nacc && a_kind[a] != ACC_SUM) {
                        const int s = farg[(f * NA + a) * B];
                        if (s < lim && s > m) m = s;
                    }
            return m;
        };
        int kj = next_join(INT_MAX), ke = next_ext(INT_MAX);
        Real lam = Real(0);
        Real Q[ADJ_MAXU] = {};
        Real G[ADJ_MAXA] = {};
        Real g_sig = Real(0), g_r = Real(0);
        int pf = nflows - 1, pft = pf >= 0 ? A.flow[pf].t : -1;
        const int nseg = (N + K - 1) / K;
#pragma unroll 1
        for (int c = nseg - 1; c >= 0; --c) {
            const int k0 = c * K;
            const int k1 = min(k0 + K, N);
            // recompute states k0 .. k0 + K and the draws of steps k0 + 1 .. k0 + K
            Real yy = ck_y[c * B];
            sy[0] = yy;
#pragma unroll 1
            for (int j = 1; j <= K; j += 4) {
                Real w4[4];
                draws4<Real>(A, keys, path, (uint64_t)(k0 + j - 1), w4);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    if (uni) {
                        yy = gbm_step(yy, ua, ub, w4[i]);
                    } else {
                        const StepRec<Real> rec = R[min(k0 + j + i, N)];  // past N: harmless states never read
                        yy = gbm_step(yy, mul_rn(pp.drift, rec.c0), mul_rn(pp.sigma, rec.c1), w4[i]);
                    }
                    sy[(j + i) * B] = yy;
                    sz[(j + i - 1) * B] = w4[i];
                }
            }
            const int jtop = (c == nseg - 1) ? k1 - k0 : k1 - k0 - 1;
            int nxt = max(max(kj, pft), ke);  // the next special step
#pragma unroll 1
            for (int j = jtop; j >= 0; --j) {
                const int k = k0 + j;
                if (k < N) {
                    Real dt = udt, sq = usq;
                    if (!uni) {
                        const StepRec<Real> rec = R[k + 1];
                        dt = rec.c0;
                        sq = rec.c1;
                    }
                    g_sig += lam * (-pp.sigma * dt + sq * sz[j * B]);
                    g_r += lam * dt;
                }
                const Real yk = sy[j * B];
                const Real Sk = spot_of<Real>(s0, yk);
                Real g = Real(0);
                if (k == nxt) {
                    if (k == kj) {  // average coefficients whose window ends here, flows in slot order
                        for (int f = 0; f < nflows; ++f)
#pragma unroll
                            for (int a = 0; a < ADJ_MAXA; ++a)
                                if (a < nacc && a_kind[a] == ACC_SUM && k == min(A.flow[f].t, a_to[a]))
                                    G[a] += fca[(f * NA + a) * B];
                        kj = next_join(k);
                    }
                    if (k == pft) {  // the flows paid at step k, in slot order
                        int f0 = pf;
                        while (f0 > 0 && A.flow[f0 - 1].t == k) --f0;
                        for (int f = f0; f <= pf; ++f) {
                            g += fcs[f * B] * Sk;
#pragma unroll
                            for (int u = 0; u < ADJ_MAXU; ++u)
                                if (u < nsu && ((A.flow[f].su_mask >> u) & 1u)) Q[u] += (Real)fP[f * B];
                        }
                        pf = f0 - 1;
                        pft = pf >= 0 ? A.flow[pf].t : -1;
                    }
                    if (k == ke) {  // running max / min: at the arg-extremum
                        for (int f = 0; f < nflows; ++f)
#pragma unroll
                            for (int a = 0; a < ADJ_MAXA; ++a)
                                if (a < nacc && a_kind[a] != ACC_SUM && farg[(f * NA + a) * B] == k)
                                    g += fca[(f * NA + a) * B] * Sk;
                        ke = next_ext(k);
                    }
                    nxt = max(max(kj, pft), ke);
                }
#pragma unroll
                for (int a = 0; a < ADJ_MAXA; ++a)  // averages: inside the window
                    if (a < nacc && a_kind[a] == ACC_SUM && k >= a_from[a]) g += G[a] * Sk;
#pragma unroll
                for (int u = 0; u < ADJ_MAXU; ++u)
                    if (u < nsu && k >= su_arm[u] && Q[u] != Real(0)) {
                        const Real x = pp.sgn[u] * (yk - pp.thr[u]) * inv_w;
                        if (x > smooth_cut<Real>()) {  // below the cut the weight is 1: no term
                            const Real sv = logistic(x);
                            const Real dls = (Real(1) - sv) * inv_w;
                            g -= Q[u] * pp.sgn[u] * dls;
                        }
                    }
#pragma unroll
                for (int a = 0; a < ADJ_MAXA; ++a)
                    if (a < nacc && a_kind[a] == ACC_SUM && k == a_from[a]) G[a] = Real(0);
                lam += g;
            }
        }
        double *o = out + A.out_off + path;
        const uint64_t n = total;
        o[8 * n] = pv_hard;
        o[0 * n] = pv;
        o[1 * n] = (double)lam / A.s0;
        o[2 * n] = (double)g_sig;
        o[3 * n] = (double)g_r - pv_t;
    }
}

template <class Real, int K, int MINB>
static const void *adj_gbm_kernel(int nsu) {
    switch (nsu) {
    case 0: return reinterpret_cast<const void *>(&k_adjoint_gbm<Real, K, 0, MINB>);
    case 1: return reinterpret_cast<const void *>(&k_adjoint_gbm<Real, K, 1, MINB>);
    default: return reinterpret_cast<const void *>(&k_adjoint_gbm<Real, K, 2, MINB>);
    }
}

// ---------------------------------------------------------------------------
// GBM sensitivities in forward (tangent) mode: one pass along the path that
// carries the derivative of the log-spot y_k in three directions D instead
// of recomputing the path for a reverse sweep. With three parameters the
// forward pass is cheaper than forward + recomputation + sweep, and it is
// the same pathwise derivative, the sweep of k_adjoint transposed term for
// term (values at rounding level apart):
//   D = 0, a uniform shift of every y_k: d/ds0 = (d/dD0) / s0 (S = s0 e^y, and
//          the barriers' log thresholds log(B / s0) move with it);
//   D = 1, sigma: dy_k += -sigma dt + sqrt(dt) z per step;
//   D = 2, r (the drift): dy_k += dt per step; the discount's -t P is added
//          at the end (d/dr moves both, as greeks.rs:70);
//   a smoothed until adds d log w / dD = sum over its weighing steps of
//          -sgn (1 - s_k) / width * dy_k/dD (s_k the step's logistic weight);
//   an average adds sum S_k dy_k/dD over its window / its count, a running
//          extremum S_k dy_k/dD at its arg-extremum;
//   a flow P = A(S, acc) w df adds df w (A_S S dy/dD + sum_a A_a dacc_a/dD +
//          A d log w / dD).
// Every primal quantity (path, spot, accumulators, weights, knock-outs, flow
// values, the hard-barrier price) is computed with k_adjoint's operations, so
// the price output is k_adjoint's bit for bit.
// ---------------------------------------------------------------------------
template <class Real, bool ACC>
__global__ void __launch_bounds__(ADJ_BLOCK) k_tangent_gbm(const AdjArgs *__restrict__ all,
                                                           const uint64_t *__restrict__ off, int n_contracts,
                                                           uint64_t total, double *__restrict__ out,
                                                           const PhiloxKeys keys) {
    for (uint64_t gp = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; gp < total;
         gp += (uint64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_contracts - 1;  // contract of global path gp
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= gp) lo = mid;
            else hi = mid - 1;
        }
        const AdjArgs &A = all[lo];
        const uint64_t path = gp - off[lo];
        const StepRec<Real> *R = reinterpret_cast<const StepRec<Real> *>(A.steps);
        const KxProgram &P = *A.P;
        const int N = A.n_times - 1;
        const AdjPar<Real> pp = adj_par<Real>(A);
        const Real s0 = pp.s0, inv_w = pp.inv_w;
        const int nflows = A.n_flows, nsu = A.n_su, nacc = ACC ? A.n_acc : 0;
        Real y = Real(0), ty = Real(0), tr = Real(0);  // y and dy/dsigma, dy/dr
        Real accraw[ADJ_MAXA], dacc[ADJ_MAXA][3];
#pragma unroll
        for (int a = 0; a < ADJ_MAXA; ++a) {
            accraw[a] = a < nacc ? (A.acc[a].kind == ACC_MAX ? Real(-INFINITY) : A.acc[a].kind == ACC_MIN ? Real(INFINITY) : Real(0)) : Real(0);
            dacc[a][0] = dacc[a][1] = dacc[a][2] = Real(0);
        }
        Real surv[ADJ_MAXU], dlw[ADJ_MAXU][3];
        int knock[ADJ_MAXU], su_arm[ADJ_MAXU];
#pragma unroll
        for (int u = 0; u < ADJ_MAXU; ++u) {
            surv[u] = Real(1);
            dlw[u][0] = dlw[u][1] = dlw[u][2] = Real(0);
            knock[u] = INT_MAX;
            su_arm[u] = u < nsu ? A.su[u].arm : INT_MAX;
        }
        double pv = 0.0, pv_t = 0.0, pv_hard = 0.0, dD[3] = {0.0, 0.0, 0.0};
        int nf = 0, nft = nflows > 0 ? A.flow[0].t : INT_MAX;
        Real z[4], vd = Real(0);  // vd: the variance slot of model_step (unused by GBM)
        for (int k = 0; k <= N; ++k) {
            if (k > 0) {
                const uint64_t d = (uint64_t)(k - 1);
                if ((d & 3u) == 0) draws4<Real>(A, keys, path, d, z);
                const Real z1 = z[d & 3u];
                const StepRec<Real> rec = R[k];
                ty += -pp.sigma * rec.c0 + rec.c1 * z1;
                tr += rec.c0;
                model_step<Real, KX_MODEL_GBM>(pp, A.scheme, rec, z1, Real(0), y, vd);
            }
            const bool pays = k == nft;
            const Real S = (ACC || pays) ? spot_of<Real>(s0, y) : Real(0);
            if (ACC)
#pragma unroll
                for (int a = 0; a < ADJ_MAXA; ++a) {
                    if (a >= nacc) continue;
                    const AdjAcc &Ac = A.acc[a];
                    if (k < Ac.i_from || k > Ac.i_to) continue;
                    if (Ac.kind == ACC_MAX || Ac.kind == ACC_MIN) {
                        if (Ac.kind == ACC_MAX ? S > accraw[a] : S < accraw[a]) {
                            accraw[a] = S;
                            dacc[a][0] = S;
                            dacc[a][1] = S * ty;
                            dacc[a][2] = S * tr;
                        }
                    } else {
                        accraw[a] = add_rn(accraw[a], S);
                        dacc[a][0] += S;
                        dacc[a][1] += S * ty;
                        dacc[a][2] += S * tr;
                    }
                }
#pragma unroll
            for (int u = 0; u < ADJ_MAXU; ++u)
                if (u < nsu && k >= su_arm[u]) {
                    const Real x = pp.sgn[u] * (y - pp.thr[u]) * inv_w;
                    if (x > smooth_cut<Real>()) {
                        const Real sv = logistic(x);
                        surv[u] *= sv;
                        const Real cdl = -pp.sgn[u] * (Real(1) - sv) * inv_w;  // d log(weight) / dy_k
                        dlw[u][0] += cdl;
                        dlw[u][1] += cdl * ty;
                        dlw[u][2] += cdl * tr;
                    }
                    if (pp.sgn[u] * y >= pp.hit[u] && knock[u] == INT_MAX) knock[u] = k;
                }
            if (!pays) continue;
            for (int f = nf; f < nflows && A.flow[f].t == k; ++f) {
                const AdjFlow &F = A.flow[f];
                nf = f + 1;
                Real accv[ADJ_MAXA], cnt[ADJ_MAXA];
#pragma unroll
                for (int a = 0; a < ADJ_MAXA; ++a) {
                    cnt[a] = Real(1);
                    accv[a] = Real(0);
                    if (a < nacc) {
                        if (A.acc[a].kind == ACC_SUM) {
                            cnt[a] = (Real)(min(k, A.acc[a].i_to) - A.acc[a].i_from + 1);
                            accv[a] = accraw[a] / cnt[a];
                        } else {
                            accv[a] = accraw[a];
                        }
                    }
                }
                Dual<Real> amt;
                if (F.kind == AK_CONST) {
                    amt.v = (Real)F.sign;
#pragma unroll
                    for (int q = 0; q < 1 + ADJ_MAXA; ++q) amt.d[q] = Real(0);
                } else {
                    amt = eval_dual<Real>(P, F.code_off, F.code_len, S, accv);
                }
                Real w = Real(1);
                Real lw[3] = {Real(0), Real(0), Real(0)};
#pragma unroll
                for (int u = 0; u < ADJ_MAXU; ++u)
                    if (u < nsu && ((F.su_mask >> u) & 1u)) {
                        w *= surv[u];
                        lw[0] += dlw[u][0];
                        lw[1] += dlw[u][1];
                        lw[2] += dlw[u][2];
                    }
                const double df = A.disc[k];
                const double fP = (double)amt.v * (double)w * df;
                pv += fP;
                pv_t += A.times[k] * fP;
                bool alive = true;
#pragma unroll
                for (int u = 0; u < ADJ_MAXU; ++u)
                    if (u < nsu && ((F.su_mask >> u) & 1u) && knock[u] <= k) alive = false;
                if (alive) pv_hard += (double)amt.v * df;
                const Real dy[3] = {Real(1), ty, tr};
#pragma unroll
                for (int D = 0; D < 3; ++D) {
                    Real g = amt.d[0] * S * dy[D];
#pragma unroll
                    for (int a = 0; a < ADJ_MAXA; ++a)
                        if (a < nacc) g += amt.d[1 + a] * (dacc[a][D] / cnt[a]);
                    dD[D] += (double)((g + amt.v * lw[D]) * w) * df;
                }
            }
            nft = nf < nflows ? A.flow[nf].t : INT_MAX;
        }
        double *o = out + A.out_off + path;
        const uint64_t n = total;
        o[8 * n] = pv_hard;
        o[0 * n] = pv;
        o[1 * n] = dD[0] / A.s0;
        o[2 * n] = dD[1];
        o[3 * n] = dD[2] - pv_t;
    }
}

template <class Real, int MODEL>
static const void *adj_kernel(bool acc) {
    return acc ? reinterpret_cast<const void *>(&k_adjoint<Real, MODEL, true>)
               : reinterpret_cast<const void *>(&k_adjoint<Real, MODEL, false>);
}

// One contract of an adjoint launch (host side).
struct AdjJob {
    AdjArgs a;                        // device pointers patched at upload
    KxProgram P;
    std::vector<unsigned char> steps;
    std::vector<double> disc, times;
    double w = 0.0;
};

static AdjJob make_adj_job(const Program &p, const Model &m, const kx_mc_config &cfg, const kx_adjoint_cfg *acfg) {
    if (cfg.flags != 0 || (cfg.rng != KX_RNG_PHILOX && cfg.rng != KX_RNG_SHARED_DRAWS) ||
        (cfg.precision != KX_PREC_FP32 && cfg.precision != KX_PREC_FP64))
        raise(KX_INVALID_ARGUMENT, "bad config");
    if (cfg.n_paths >= (1ull << 32)) raise(KX_INVALID_ARGUMENT, "n_paths must be below 2^32");
    validate_model(m);
    if (!(m.s0 > 0.0)) raise(KX_UNSUPPORTED, "adjoint: s0 must be positive");
    auto grid = time_grid_forced(p.plan, cfg.steps_per_year, m.requires_fine_grid());
    validate_grid(grid);
    const int n = (int)grid.size();
    const int N = n - 1;
    AdjJob J;
    StepTables tab;
    bind(p.low, grid, m, cfg.rate, J.P, tab);
    AdjArgs &a = J.a;
    memset(&a, 0, sizeof a);
    schedule(p.low, J.P, tab, m, a);
    uint32_t K = acfg && acfg->checkpoint_every ? acfg->checkpoint_every : 16u;
    K = (K + 3) / 4 * 4;
    if (K > (uint32_t)ADJ_KMAX) K = ADJ_KMAX;
    while ((N + (int)K - 1) / (int)K + 1 > ADJ_MAXCK && K < (uint32_t)ADJ_KMAX) K += 4;
    if ((N + (int)K - 1) / (int)K + 1 > ADJ_MAXCK) raise(KX_UNSUPPORTED, "adjoint: grid too long for the checkpoint store");
    a.K = (int)K;
    // smoothing width: default 0.5 * sigma_eff * sqrt(mean dt)
    double w = acfg ? acfg->smoothing_width : 0.0;
    const double dtm = N > 0 ? grid.back() / N : 1.0;
    if (!(w > 0.0)) {
        const double se = m.kind == KX_MODEL_GBM ? m.sigma : std::sqrt(std::max(m.v0, m.theta));
        w = 0.5 * std::max(se, 1e-8) * std::sqrt(dtm);
    }
    J.w = w;
    a.inv_w = 1.0 / w;
    a.n_times = n;
    a.model = m.kind;
    a.scheme = m.scheme;
    a.n_paths = cfg.n_paths;
    a.seed = cfg.seed;
    a.s0 = m.s0;
    a.mu = m.kind == KX_MODEL_GBM ? m.mu : m.r;
    a.sigma = m.sigma;
    a.v0 = m.v0; a.kappa = m.kappa; a.theta = m.theta; a.sigma_v = m.sigma_v; a.rho = m.rho;
    a.rho_perp = std::sqrt(std::max(1.0 - m.rho * m.rho, 0.0));
    a.r = m.r;
    const bool f64 = cfg.precision == KX_PREC_FP64;
    // uniform grid: every step's (dt, sqrt dt) equal in the launch precision
    const bool f64p = cfg.precision == KX_PREC_FP64;
    a.uniform = N >= 1 ? 1 : 0;
    a.uc0 = N >= 1 ? grid[1] - grid[0] : 0.0;
    a.uc1 = std::sqrt(a.uc0);
    for (int k = 2; k <= N && a.uniform; ++k) {
        const double dt = grid[k] - grid[k - 1], sq = std::sqrt(dt);
        if (f64p ? (dt != a.uc0 || sq != a.uc1) : ((float)dt != (float)a.uc0 || (float)sq != (float)a.uc1))
            a.uniform = 0;
    }
    J.steps.resize(n * (f64 ? sizeof(StepRec<double>) : sizeof(StepRec<float>)));
    for (int k = 0; k < n; ++k) {
        const double dt = k == 0 ? 0.0 : grid[k] - grid[k - 1];
        if (f64) reinterpret_cast<StepRec<double> *>(J.steps.data())[k] = {dt, std::sqrt(dt), 0u, 0u};
        else reinterpret_cast<StepRec<float> *>(J.steps.data())[k] = {(float)dt, (float)std::sqrt(dt), 0u, 0u};
    }
    J.disc = tab.disc;
    J.times = grid;
    return J;
}

// Launch the adjoint over `jobs` (one model kind, one precision); returns the
// statistics of the ADJ_OUT per-path outputs of every contract.
static std::vector<std::vector<Stats>> run_adjoint(Ctx &c, std::vector<AdjJob> &jobs, bool f64, int model, int rng) {
    const int nc = (int)jobs.size();
    std::vector<KxProgram> progs;
    std::vector<unsigned char> steps;
    std::vector<double> dt;  // disc then times, per contract
    std::vector<uint64_t> off(nc + 1, 0);
    std::vector<size_t> soff(nc), doff(nc);
    for (int i = 0; i < nc; ++i) {
        progs.push_back(jobs[i].P);
        soff[i] = steps.size();
        steps.insert(steps.end(), jobs[i].steps.begin(), jobs[i].steps.end());
        doff[i] = dt.size();
        dt.insert(dt.end(), jobs[i].disc.begin(), jobs[i].disc.end());
        dt.insert(dt.end(), jobs[i].times.begin(), jobs[i].times.end());
        off[i + 1] = off[i] + jobs[i].a.n_paths;
    }
    const uint64_t total = off[nc];
    c.progs.ensure(progs.size() * sizeof(KxProgram));
    c.steps.ensure(steps.size());
    c.disc.ensure(dt.size() * sizeof(double));
    c.cons.ensure(nc * sizeof(AdjArgs));
    c.items.ensure((nc + 1) * sizeof(uint64_t));
    c.pv.ensure(std::max<uint64_t>(1, total) * ADJ_OUT * sizeof(double));
    std::vector<AdjArgs> args(nc);
    for (int i = 0; i < nc; ++i) {
        AdjArgs a = jobs[i].a;
        a.P = c.progs.as<KxProgram>() + i;
        a.steps = c.steps.as<unsigned char>() + soff[i];
        a.disc = c.disc.as<double>() + doff[i];
        a.times = c.disc.as<double>() + doff[i] + jobs[i].disc.size();
        a.out_off = off[i];
        if (rng == KX_RNG_SHARED_DRAWS) {
            DrawStore &ds = c.draws;
            if (!ds.set) raise(KX_INVALID_ARGUMENT, "no shared draws registered");
            const int N = a.n_times - 1;
            if (ds.n_paths < a.n_paths || ds.dpp < (uint64_t)N * (model == KX_MODEL_HESTON ? 2 : 1))
                raise(KX_INVALID_ARGUMENT, "shared draws too small for this simulation");
            a.z64 = ds.is64 ? ds.z64.as<double>() : nullptr;
            a.z32 = ds.is64 ? nullptr : ds.z32.as<float>();
            a.z_dpp = ds.dpp;
        }
        args[i] = a;
    }
    KX_CUDA(cudaMemcpyAsync(c.progs.p, progs.data(), progs.size() * sizeof(KxProgram), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemcpyAsync(c.steps.p, steps.data(), steps.size(), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemcpyAsync(c.disc.p, dt.data(), dt.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemcpyAsync(c.cons.p, args.data(), nc * sizeof(AdjArgs), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemcpyAsync(c.items.p, off.data(), (nc + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, c.stream));
    c.last.h2d_bytes += progs.size() * sizeof(KxProgram) + steps.size() + dt.size() * sizeof(double) +
                        nc * sizeof(AdjArgs) + (nc + 1) * sizeof(uint64_t);
    bool acc = false;
    int max_n = 0, nsu = -1;
    bool same_nsu = true;
    for (auto &j : jobs) {
        acc |= j.a.n_acc > 0;
        max_n = std::max(max_n, j.a.n_times - 1);
        if (nsu >= 0 && j.a.n_su != nsu) same_nsu = false;
        nsu = j.a.n_su;
    }
    const void *kfn = model == KX_MODEL_GBM
                          ? (f64 ? adj_kernel<double, KX_MODEL_GBM>(acc) : adj_kernel<float, KX_MODEL_GBM>(acc))
                          : (f64 ? adj_kernel<double, KX_MODEL_HESTON>(acc) : adj_kernel<float, KX_MODEL_HESTON>(acc));
    // GBM: the specialised kernels, tuned over checkpoint interval and register
    // budget on the call's own work (results do not depend on the choice: every
    // GBM kernel repeats k_adjoint's operations in its order, and the
    // recomputation repeats the forward pass's). KX_ADJOINT_KERNEL = "general"
    // keeps the generic kernel.
    std::vector<std::pair<int, const void *>> cands;
    int kck = 0;  // checkpoint interval of the chosen GBM kernel (0: the generic kernel)
    const char *kenv = getenv("KX_ADJOINT_KERNEL");
    const bool generic_only = kenv && strcmp(kenv, "general") == 0;
    const bool tangent_only = kenv && strcmp(kenv, "tangent") == 0;
    // GBM: the forward-mode kernel (one pass, no recomputation) is timed beside the reverse
    // kernels; KX_ADJOINT_KERNEL = "tangent" keeps it, KX_ADJOINT_CANDIDATE picks among the
    // reverse kernels only (those give k_adjoint's values bit for bit)
    const void *tan_fn = nullptr;
    if (model == KX_MODEL_GBM && !generic_only)
        tan_fn = f64 ? (acc ? (const void *)&k_tangent_gbm<double, true> : (const void *)&k_tangent_gbm<double, false>)
                     : (acc ? (const void *)&k_tangent_gbm<float, true> : (const void *)&k_tangent_gbm<float, false>);
    bool use_tan = false;
    if (model == KX_MODEL_GBM && !acc && same_nsu && !generic_only) {
        // the register-resident kernel at two register budgets (resident blocks per SM)
        if (max_n / 8 + 1 <= ADJ_MAXCK) {
            cands.push_back({8, f64 ? adj_gbm_kernel<double, 8, 4>(nsu) : adj_gbm_kernel<float, 8, 8>(nsu)});
            cands.push_back({8, f64 ? adj_gbm_kernel<double, 8, 2>(nsu) : adj_gbm_kernel<float, 8, 5>(nsu)});
        }
        if (max_n / 16 + 1 <= ADJ_MAXCK) {
            cands.push_back({16, f64 ? adj_gbm_kernel<double, 16, 4>(nsu) : adj_gbm_kernel<float, 16, 8>(nsu)});
            cands.push_back({16, f64 ? adj_gbm_kernel<double, 16, 2>(nsu) : adj_gbm_kernel<float, 16, 5>(nsu)});
        }
    }
    // the accumulator kernel at two register budgets (resident blocks per SM), specialised where
    // every contract of the launch has one accumulator of one kind and no smoothed barrier, or
    // none and the same number (0 or 1) of smoothed barriers
    int one_kind = -1;
    if (model == KX_MODEL_GBM) {
        one_kind = jobs[0].a.n_acc == 1 && jobs[0].a.n_su == 0 ? jobs[0].a.acc[0].kind : -1;
        for (auto &j : jobs)
            if (j.a.n_acc != 1 || j.a.n_su != 0 || j.a.acc[0].kind != one_kind) one_kind = -1;
    }
    const void *acc_fns[2];
    if (!acc && same_nsu && nsu >= 0 && nsu <= 1) {  // no accumulators, 0 or 1 smoothed barriers
        acc_fns[0] = f64 ? (nsu ? (const void *)&k_adjoint_gbm_acc<double, 3, 0, -1, 1>
                                : (const void *)&k_adjoint_gbm_acc<double, 3, 0, -1, 0>)
                         : (nsu ? (const void *)&k_adjoint_gbm_acc<float, 6, 0, -1, 1>
                                : (const void *)&k_adjoint_gbm_acc<float, 6, 0, -1, 0>);
        acc_fns[1] = f64 ? (nsu ? (const void *)&k_adjoint_gbm_acc<double, 2, 0, -1, 1>
                                : (const void *)&k_adjoint_gbm_acc<double, 2, 0, -1, 0>)
                         : (nsu ? (const void *)&k_adjoint_gbm_acc<float, 8, 0, -1, 1>
                                : (const void *)&k_adjoint_gbm_acc<float, 8, 0, -1, 0>);
    } else if (one_kind == ACC_SUM) {
        acc_fns[0] = f64 ? (const void *)&k_adjoint_gbm_acc<double, 3, 1, ACC_SUM, 0>
                         : (const void *)&k_adjoint_gbm_acc<float, 6, 1, ACC_SUM, 0>;
        acc_fns[1] = f64 ? (const void *)&k_adjoint_gbm_acc<double, 2, 1, ACC_SUM, 0>
                         : (const void *)&k_adjoint_gbm_acc<float, 8, 1, ACC_SUM, 0>;
    } else if (one_kind == ACC_MAX || one_kind == ACC_MIN) {
        const bool mx = one_kind == ACC_MAX;
        acc_fns[0] = f64 ? (mx ? (const void *)&k_adjoint_gbm_acc<double, 3, 1, ACC_MAX, 0>
                               : (const void *)&k_adjoint_gbm_acc<double, 3, 1, ACC_MIN, 0>)
                         : (mx ? (const void *)&k_adjoint_gbm_acc<float, 6, 1, ACC_MAX, 0>
                               : (const void *)&k_adjoint_gbm_acc<float, 6, 1, ACC_MIN, 0>);
        acc_fns[1] = f64 ? (mx ? (const void *)&k_adjoint_gbm_acc<double, 2, 1, ACC_MAX, 0>
                               : (const void *)&k_adjoint_gbm_acc<double, 2, 1, ACC_MIN, 0>)
                         : (mx ? (const void *)&k_adjoint_gbm_acc<float, 8, 1, ACC_MAX, 0>
                               : (const void *)&k_adjoint_gbm_acc<float, 8, 1, ACC_MIN, 0>);
    } else {
        acc_fns[0] = f64 ? (const void *)&k_adjoint_gbm_acc<double, 3> : (const void *)&k_adjoint_gbm_acc<float, 6>;
        acc_fns[1] = f64 ? (const void *)&k_adjoint_gbm_acc<double, 2> : (const void *)&k_adjoint_gbm_acc<float, 4>;
    }
    if (model == KX_MODEL_GBM && !generic_only)
        for (const void *fn : acc_fns)
            for (int kc : {8, 16, 32}) cands.push_back({kc, fn});
    if (total > 0) {
        const AdjArgs *ap = c.cons.as<AdjArgs>();
        const uint64_t *op = c.items.as<uint64_t>();
        double *outp = c.pv.as<double>();
        PhiloxKeys keys{};
        bool one_seed = true;
        for (int i = 0; i < nc; ++i) one_seed = one_seed && args[i].seed == args[0].seed;
        if (one_seed) keys = philox_keys(args[0].seed);
        int n_ck = 0;  // checkpoint rows of the GBM kernels (set per candidate)
        AdjSmem lay{0, 0, 0, 0};  // shared-memory records of the accumulator kernel (set per candidate)
        for (auto &j : jobs) {
            lay.nf = std::max(lay.nf, j.a.n_flows);
            lay.na = std::max(lay.na, j.a.n_acc);
        }
        void *kargs_g[] = {&ap, &op, (void *)&nc, (void *)&total, &outp, &keys};
        void *kargs_r[] = {&ap, &op, (void *)&nc, (void *)&total, &outp, &keys, (void *)&n_ck};
        void *kargs_a[] = {&ap, &op, (void *)&nc, (void *)&total, &outp, &keys, (void *)&lay};
        auto launch = [&](const void *fn, int ck_every) {
            // the GBM kernels keep checkpoints and flow records in shared memory
            size_t smem = 0;
            const bool is_acc = ck_every > 0 && (fn == acc_fns[0] || fn == acc_fns[1]);
            if (is_acc) {
                lay.K = ck_every;
                lay.n_ck = max_n / ck_every + 1;
                smem = f64 ? adj_smem_bytes<double>(lay) : adj_smem_bytes<float>(lay);
                KX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            } else if (ck_every > 0) {
                n_ck = max_n / ck_every + 1;
                const size_t real = f64 ? 8 : 4;
                smem = (size_t)ADJ_BLOCK * (ADJ_MAXF * sizeof(double) + (ADJ_MAXF + n_ck) * real);
                KX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            }
            const int full = persistent_blocks(fn, ADJ_BLOCK, smem);
            const int blocks = (int)std::min<uint64_t>((uint64_t)full, (total + ADJ_BLOCK - 1) / ADJ_BLOCK);
            KX_CUDA(cudaEventRecord(c.ev0, c.stream));
            KX_CUDA(cudaLaunchKernel(fn, dim3(blocks), dim3(ADJ_BLOCK), is_acc ? kargs_a : ck_every > 0 ? kargs_r : kargs_g,
                                     smem, c.stream));
            KX_CUDA(cudaEventRecord(c.ev1, c.stream));
            KX_CUDA(cudaEventSynchronize(c.ev1));
            float ms = 0.f;
            KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
            c.last.grid_blocks = (uint32_t)blocks;
            return ms;
        };
        if (!cands.empty()) {
            // the chosen candidate (index + 1; cands.size() + 1: the tangent kernel) per
            // precision, accumulators present and barrier count (ADJ_MAXU + 1: mixed); 0: not
            // tuned yet (default: the first with K = 16)
            static int tuned[2][2][ADJ_MAXU + 2] = {};
            const char *env = getenv("KX_TUNE");
            const bool tune = !(env && env[0] == '0');
            int &tk = tuned[f64 ? 1 : 0][acc ? 1 : 0][same_nsu ? std::min(std::max(nsu, 0), ADJ_MAXU) : ADJ_MAXU + 1];
            if (tune && tk == 0 && cands.size() + (tan_fn ? 1 : 0) > 1) {
                float best = 1e30f;
                const char *vb = getenv("KX_TUNE_VERBOSE");
                for (size_t q = 0; q < cands.size() + (tan_fn ? 1 : 0); ++q) {
                    // this call's own work: every candidate computes it
                    const bool t = q == cands.size();
                    const float ms = t ? launch(tan_fn, 0) : launch(cands[q].second, cands[q].first);
                    if (ms < best) { best = ms; tk = (int)q + 1; }
                    if (vb && vb[0] == '1')
                        fprintf(stderr, "[kx adjoint tune] candidate %zu (%s K %d): %.3f ms\n", q,
                                t ? "tangent" : "reverse", t ? 0 : cands[q].first, ms);
                }
            }
            size_t pick = 0;
            if (tk > 0 && (size_t)tk <= cands.size()) pick = (size_t)tk - 1;
            else
                for (size_t q = cands.size(); q-- > 0;)
                    if (cands[q].first == 16) pick = q;
            use_tan = tan_fn && tk == (int)cands.size() + 1;
            const char *ce = getenv("KX_ADJOINT_CANDIDATE");  // a given reverse candidate (tests: each gives the same values)
            if (ce && ce[0]) {
                pick = (size_t)atoi(ce) % cands.size();
                use_tan = false;
            }
            kfn = cands[pick].second;
            kck = cands[pick].first;
        } else if (tan_fn) {  // accumulators or mixed barrier counts: the generic kernel or the tangent one
            static int tuned_g[2][2] = {};  // 1: generic, 2: tangent; 0: not tuned yet
            const char *env = getenv("KX_TUNE");
            int &tg = tuned_g[f64 ? 1 : 0][acc ? 1 : 0];
            if (!(env && env[0] == '0') && tg == 0) {
                const float mg = launch(kfn, 0), mt = launch(tan_fn, 0);
                tg = mt < mg ? 2 : 1;
            }
            use_tan = tg == 2;
        }
        if (tangent_only && tan_fn) use_tan = true;
        if (use_tan) {
            kfn = tan_fn;
            kck = 0;
        }
        const float ms = launch(kfn, kck);
        c.last.kernel_ms += ms;
        c.last.kernel_launches++;
        c.last.block_threads = ADJ_BLOCK;
    }
    // the output rows a model fills: GBM price, d/ds0, d/dsigma, d/dr and the hard-barrier price
    // (rows 4..7 are Heston's); the others stay empty statistics
    std::vector<int> rows;
    for (int q = 0; q < ADJ_OUT; ++q)
        if (model != KX_MODEL_GBM || q <= 3 || q == 8) rows.push_back(q);
    std::vector<StatsJob> sj;
    for (int i = 0; i < nc; ++i) {
        c.last.path_steps += jobs[i].a.n_paths * (uint64_t)(jobs[i].a.n_times - 1);
        c.last.steps_simulated += (use_tan ? 1 : 2) * jobs[i].a.n_paths * (uint64_t)(jobs[i].a.n_times - 1);  // forward (+ recompute)
        for (int q : rows) {
            StatsJob j;
            j.begin = (uint64_t)q * total + off[i];
            j.n = jobs[i].a.n_paths;
            sj.push_back(j);
        }
    }
    auto st = device_stats(c, c.pv.as<double>(), 0, sj);
    std::vector<std::vector<Stats>> res(nc);
    for (int i = 0; i < nc; ++i) {
        res[i].assign(ADJ_OUT, Stats{});
        for (size_t r = 0; r < rows.size(); ++r) res[i][rows[r]] = st[(size_t)i * rows.size() + r];
    }
    return res;
}

static void fill_sens(const std::vector<Stats> &st, int model, double w, kx_sens *out) {
    auto R = [&](int q) { return finish(st[q]); };
    memset(out, 0, sizeof *out);
    out->price = R(0).price;
    out->price_se = R(0).std_error;
    out->d_s0 = R(1).price;
    out->se_s0 = R(1).std_error;
    out->smoothing_width = w;
    if (model == KX_MODEL_GBM) {
        out->d_sigma = R(2).price; out->se_sigma = R(2).std_error;
        out->d_r = R(3).price; out->se_r = R(3).std_error;
    } else {
        out->d_v0 = R(2).price; out->se_v0 = R(2).std_error;
        out->d_r = R(3).price; out->se_r = R(3).std_error;
        out->d_kappa = R(4).price; out->se_kappa = R(4).std_error;
        out->d_theta = R(5).price; out->se_theta = R(5).std_error;
        out->d_sigma_v = R(6).price; out->se_sigma_v = R(6).std_error;
        out->d_rho = R(7).price; out->se_rho = R(7).std_error;
    }
}

// Portfolio pricing with per-contract pathwise sensitivities: one adjoint
// launch per (model kind, precision) group; prices use the hard barriers.
void portfolio_adjoint(Ctx &c, size_t n, const kx_program *const *progs, const kx_model *models,
                       const kx_mc_config *cfgs, kx_price_result *out, kx_sens *sens) {
    std::vector<AdjJob> all;
    for (size_t i = 0; i < n; ++i) {
        if (cfgs[i].rng != KX_RNG_PHILOX) raise(KX_UNSUPPORTED, "portfolio pricing uses Philox normals");
        all.push_back(make_adj_job(program_of(progs[i]), model_from_c(&models[i]), cfgs[i], nullptr));
    }
    // one launch per (model kind, precision, averages or extrema present,
    // smoothed barrier count): each group gets the kernel specialised for it
    for (int kind = 0; kind < 2; ++kind)
        for (int prec = 0; prec < 2; ++prec)
            for (int acc = 0; acc < 2; ++acc)
                for (int nsu = 0; nsu <= ADJ_MAXU; ++nsu) {
                std::vector<size_t> idx;
                for (size_t i = 0; i < n; ++i)
                    if (models[i].kind == kind && cfgs[i].precision == prec && (all[i].a.n_acc > 0) == (acc == 1) &&
                        all[i].a.n_su == nsu)
                        idx.push_back(i);
                if (idx.empty()) continue;
                std::vector<AdjJob> jobs;
                for (size_t i : idx) jobs.push_back(all[i]);
                auto st = run_adjoint(c, jobs, prec == KX_PREC_FP64, kind, KX_RNG_PHILOX);
                for (size_t q = 0; q < idx.size(); ++q) {
                    out[idx[q]] = finish(st[q][8]);
                    fill_sens(st[q], kind, jobs[q].w, &sens[idx[q]]);
                }
                }
}

}  // namespace kx

using namespace kx;

extern "C" kx_status kx_greeks_adjoint(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg,
                                       const kx_adjoint_cfg *acfg, kx_sens *out) {
    return guarded([&] {
        const Program &p = program_of(prog);
        Model m = model_from_c(model);
        if (!cfg || !out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        std::vector<AdjJob> jobs;
        jobs.push_back(make_adj_job(p, m, *cfg, acfg));
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        auto st = run_adjoint(c, jobs, cfg->precision == KX_PREC_FP64, m.kind, cfg->rng);
        fill_sens(st[0], m.kind, jobs[0].w, out);
        c.last.total_ms += now_ms();
    });
}
