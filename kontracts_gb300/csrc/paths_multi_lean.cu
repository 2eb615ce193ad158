// paths_multi_lean.cu — the path kernel of correlated multi-factor GBM
// (CorrelatedGbmN, multi_asset.rs:107-170) for contracts whose conditions and
// amounts are affine in the factor spots: baskets and spreads, European or
// Bermudan, with knock-out barriers on one factor or on a basket.
//
// The general kernel (k_paths<.., M_MULTI>) interprets the contract's postfix
// programs through its event handler at every step, with the factor state in
// local arrays. Here the host compiles the contract once more:
//  * the condition of every until that reads prices, c(S) cmp 0 with c
//    affine in the spots (c0 + sum_i a_i S_i), becomes a barrier row;
//  * every flow amount becomes sign * f(c0 + sum_i a_i S_i), f the identity,
//    max(., K) or min(., K): a call or put on a basket or a spread;
//  * the time conditions become a fixed list of event steps (arming of the
//    barriers, payment of the flows), as in the static schedules of k_lean.
// Per step a lane draws the factors' normals, correlates them with the
// Cholesky factor and steps every log-spot; the spots and the affine forms
// are evaluated only when a barrier is live or a flow is due. Knock-outs come
// before the event of the same step and flows are added in slot order, as
// cashflows / present_value do (pricer.rs:374-433).
//
// Draws: step k of path p takes normals (k - 1) n .. (k - 1) n + n - 1 of the
// path's Philox stream (n factors, four normals per block), as the general
// kernel does. A lane advances ML_RS = 4 steps per round, which take exactly
// n Philox blocks, so where each block starts is known at compile time.
//
// An affine form adds its terms in another order than the interpreter (a
// basket (S1 + ... + Sn) / n - K becomes -K + S1 / n + ... + Sn / n), so a
// path's value agrees with the general kernel's to rounding, not bit for bit.
#include <cmath>
#include <cstring>
#include <map>

#include "launch.hpp"

namespace kx {

constexpr int ML_BLOCK = 128;
constexpr int ML_RS = 4;       // grid steps per round
constexpr int ML_MAXB = 4;     // affine barriers
constexpr int ML_MAXF = 8;     // flows
constexpr int ML_MAXEV = 64;   // event steps
constexpr int ML_CHUNK = 64;   // paths a warp takes from the launch counter at a time

enum : uint8_t { MF_AFFINE = 0, MF_MAX = 1, MF_MIN = 2, MF_CONST = 3 };

struct MultiLeanArgs {
    const void *steps;                   // StepRec<Real>[n_times]
    const double *disc;                  // discount factor of each step
    double *pv;                          // pv[i]: path path_base + i
    unsigned long long *next;            // paths handed out
    unsigned long long *steps_done;      // path steps simulated
    uint64_t n_paths;
    uint32_t path_base, stream;
    int32_t n_times, uniform, n_ev;
    uint32_t all_flows;
    double uc0, uc1;
    float uc0f, uc1f;
    uint32_t rk[20];                     // Philox round keys of the seed
    double s0[KX_MAX_NS], drift[KX_MAX_NS], sigma[KX_MAX_NS];
    float s0f[KX_MAX_NS], driftf[KX_MAX_NS], sigmaf[KX_MAX_NS];
    double chol[KX_MAX_NS * (KX_MAX_NS + 1) / 2];
    float cholf[KX_MAX_NS * (KX_MAX_NS + 1) / 2];
    int32_t ev_step[ML_MAXEV];
    uint8_t ev_arm[ML_MAXEV];            // barriers armed (and tested) at the step
    uint8_t ev_pay[ML_MAXEV];            // flows paid at the step unless knocked out
    uint8_t kill[ML_MAXB];               // flows dropped when the barrier knocks
    uint8_t b_cmp[ML_MAXB];              // KxCmp of "form cmp 0"
    uint8_t f_form[ML_MAXF];
    uint8_t f_neg;                       // flows whose sign is negative
    uint8_t pad[3];
    double b_c[ML_MAXB][KX_MAX_NS + 1];  // [0] constant, [1 + i] coefficient of S_i
    float b_cf[ML_MAXB][KX_MAX_NS + 1];
    double f_c[ML_MAXF][KX_MAX_NS + 1];
    float f_cf[ML_MAXF][KX_MAX_NS + 1];
    double f_k[ML_MAXF];                 // K of max / min forms; the amount of a constant flow
    float f_kf[ML_MAXF];
    double f_sign[ML_MAXF];
};
static_assert(sizeof(MultiLeanArgs) <= 4000, "kernel parameters");

template <class Real, int NA>
__device__ __forceinline__ Real affine(const double (&c)[KX_MAX_NS + 1], const float (&cf)[KX_MAX_NS + 1],
                                       const Real (&S)[NA]) {
    Real v = pick<Real>(c[0], cf[0]);
#pragma unroll
    for (int i = 0; i < NA; ++i) v = v + pick<Real>(c[1 + i], cf[1 + i]) * S[i];
    return v;
}

template <class Real, int NA>
__device__ __forceinline__ bool barrier_hit(const MultiLeanArgs &A, int b, const Real (&S)[NA]) {
    const Real v = affine<Real, NA>(A.b_c[b], A.b_cf[b], S);
    switch (A.b_cmp[b]) {
    case CMP_GE: return v >= Real(0);
    case CMP_GT: return v > Real(0);
    case CMP_LE: return v <= Real(0);
    default: return v < Real(0);
    }
}

// The contract at step k: knock-outs of the live barriers, then the event of
// the step if one is due (barriers armed and tested at once, flows paid).
template <class Real, int NA>
__device__ __forceinline__ void multi_event(const MultiLeanArgs &A, const Real (&S)[NA], int k, bool at_ev,
                                            uint32_t &live, uint32_t &rem, int &e, double &pv) {
#pragma unroll
    for (int b = 0; b < ML_MAXB; ++b)
        if (((live >> b) & 1u) && barrier_hit<Real, NA>(A, b, S)) {
            live &= ~(1u << b);
            rem &= ~(uint32_t)A.kill[b];
        }
    if (!at_ev) return;
    const uint32_t arm = A.ev_arm[e];
#pragma unroll
    for (int b = 0; b < ML_MAXB; ++b)
        if ((arm >> b) & 1u) {
            if (barrier_hit<Real, NA>(A, b, S)) rem &= ~(uint32_t)A.kill[b];
            else live |= 1u << b;
        }
    const uint32_t pay = A.ev_pay[e] & rem;
    if (pay) {
        const double D = A.disc[k];
#pragma unroll
        for (int f = 0; f < ML_MAXF; ++f)
            if ((pay >> f) & 1u) {
                double amt;
                if (A.f_form[f] == MF_CONST) {
                    amt = A.f_k[f];
                } else {
                    Real v = affine<Real, NA>(A.f_c[f], A.f_cf[f], S);
                    const Real K = pick<Real>(A.f_k[f], A.f_kf[f]);
                    if (A.f_form[f] == MF_MAX) v = fmax(v, K);
                    else if (A.f_form[f] == MF_MIN) v = fmin(v, K);
                    amt = (double)(((A.f_neg >> f) & 1u) ? -v : v);
                }
                pv = __dadd_rn(pv, __dmul_rn(amt, D));
            }
    }
    rem &= ~(uint32_t)A.ev_pay[e];
    ++e;
}

template <class Real, int NA>
__device__ __forceinline__ void spots(const MultiLeanArgs &A, const Real (&ym)[NA], Real (&S)[NA]) {
#pragma unroll
    for (int i = 0; i < NA; ++i) S[i] = spot_of<Real>(pick<Real>(A.s0[i], A.s0f[i]), ym[i]);
}

template <class Real, int NA>
__global__ void __launch_bounds__(ML_BLOCK, sizeof(Real) == 4 ? 8 : 4)
    k_multi_lean(const __grid_constant__ MultiLeanArgs A) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const StepRec<Real> *R = static_cast<const StepRec<Real> *>(A.steps);
    const int nt = A.n_times;

    uint64_t nx = 0, end = 0;  // the warp's chunk of paths
    bool drained = false;
    int64_t path = -1;         // local path index, -1 when the lane is idle
    int k = 1;
    Real ym[NA];
    uint32_t live = 0, rem = 0;
    int e = 0;
    double pv = 0.0;
    uint32_t my_steps = 0;

    while (true) {
        // ---- hand paths to idle lanes (warp-uniform control) ----
        unsigned idle = __ballot_sync(FULL, path < 0);
        while (idle) {
            if (nx >= end) {
                if (drained) break;
                unsigned long long c0 = 0;
                if (lane == 0) c0 = atomicAdd(A.next, (unsigned long long)ML_CHUNK);
                c0 = __shfl_sync(FULL, c0, 0);
                if (c0 >= A.n_paths) {
                    drained = true;
                    break;
                }
                nx = c0;
                end = c0 + ML_CHUNK < A.n_paths ? c0 + ML_CHUNK : A.n_paths;
            }
            const uint32_t avail = (uint32_t)(end - nx);
            const int nidle = __popc(idle);
            const int take = avail < (uint32_t)nidle ? (int)avail : nidle;
            const int rank = __popc(idle & lt);
            if (path < 0 && rank < take) {
                path = (int64_t)(nx + (uint64_t)rank);
                // state at t = 0 (S = s0), then the contract at step 0
                Real S[NA];
#pragma unroll
                for (int i = 0; i < NA; ++i) {
                    ym[i] = Real(0);
                    S[i] = pick<Real>(A.s0[i], A.s0f[i]);
                }
                live = 0u;
                rem = A.all_flows;
                e = 0;
                pv = 0.0;
                multi_event<Real, NA>(A, S, 0, A.n_ev > 0 && A.ev_step[0] == 0, live, rem, e, pv);
                k = 1;
                if (nt <= 1 || rem == 0u) {
                    A.pv[path] = pv;
                    path = -1;
                }
            }
            nx += (uint64_t)take;
            idle = __ballot_sync(FULL, path < 0);
        }
        if (__ballot_sync(FULL, path >= 0) == 0u) {
            if (drained) break;
            continue;
        }

        // ---- one round: steps k .. k + 3 of busy lanes ((k - 1) is a multiple of 4) ----
        if (path >= 0) {
            const uint64_t pg = (uint64_t)A.path_base + (uint64_t)path;
            const uint32_t blk0 = (uint32_t)((k - 1) / ML_RS) * (uint32_t)NA;
            Real zz[4] = {Real(0), Real(0), Real(0), Real(0)};
            bool alive = true;
#pragma unroll
            for (int j = 0; j < ML_RS; ++j) {
                const int kk = k + j;
                if (alive && kk < nt) {
                    Real z[NA];
#pragma unroll
                    for (int i = 0; i < NA; ++i) {
                        const int q = j * NA + i;  // draw of the round (compile-time)
                        if ((q & 3) == 0) {
                            const uint4 w = philox4x32_10_rk(
                                make_uint4(blk0 + (uint32_t)(q >> 2), (uint32_t)pg, (uint32_t)(pg >> 32), A.stream),
                                A.rk);
                            box_muller(w.x, w.y, zz[0], zz[1]);
                            box_muller(w.z, w.w, zz[2], zz[3]);
                        }
                        z[i] = zz[q & 3];
                    }
                    Real c0, c1;
                    if (A.uniform) {
                        c0 = pick<Real>(A.uc0, A.uc0f);
                        c1 = pick<Real>(A.uc1, A.uc1f);
                    } else {
                        const StepRec<Real> rec = R[kk];
                        c0 = rec.c0;
                        c1 = rec.c1;
                    }
                    // w = L z (multi_asset.rs:146-156), then each factor's exact log step
#pragma unroll
                    for (int i = 0; i < NA; ++i) {
                        Real wi = Real(0);
                        const int row = i * (i + 1) / 2;
#pragma unroll
                        for (int jj = 0; jj <= i; ++jj) wi = wi + pick<Real>(A.chol[row + jj], A.cholf[row + jj]) * z[jj];
                        ym[i] = gbm_step(ym[i], pick<Real>(A.drift[i], A.driftf[i]) * c0,
                                         pick<Real>(A.sigma[i], A.sigmaf[i]) * c1, wi);
                    }
                    ++my_steps;
                    const bool at_ev = e < A.n_ev && A.ev_step[e] == kk;
                    if (live || at_ev) {
                        Real S[NA];
                        spots<Real, NA>(A, ym, S);
                        multi_event<Real, NA>(A, S, kk, at_ev, live, rem, e, pv);
                        alive = rem != 0u;
                    }
                }
            }
            k += ML_RS;
            if (!alive || k >= nt) {
                A.pv[path] = pv;
                path = -1;
            }
        }
    }
    unsigned long long tot = (unsigned long long)my_steps;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
    if (lane == 0 && tot) atomicAdd(A.steps_done, tot);
}

#define KX_ML(R, N) template __global__ void k_multi_lean<R, N>(const __grid_constant__ MultiLeanArgs);
KX_ML(float, 2) KX_ML(float, 3) KX_ML(float, 4) KX_ML(float, 5) KX_ML(float, 6) KX_ML(float, 7)
KX_ML(double, 2) KX_ML(double, 3) KX_ML(double, 4) KX_ML(double, 5) KX_ML(double, 6) KX_ML(double, 7)
#undef KX_ML

static const void *multi_lean_kernel(bool f64, int na) {
    static const void *const k32[] = {(const void *)&k_multi_lean<float, 2>, (const void *)&k_multi_lean<float, 3>,
                                      (const void *)&k_multi_lean<float, 4>, (const void *)&k_multi_lean<float, 5>,
                                      (const void *)&k_multi_lean<float, 6>, (const void *)&k_multi_lean<float, 7>};
    static const void *const k64[] = {(const void *)&k_multi_lean<double, 2>, (const void *)&k_multi_lean<double, 3>,
                                      (const void *)&k_multi_lean<double, 4>, (const void *)&k_multi_lean<double, 5>,
                                      (const void *)&k_multi_lean<double, 6>, (const void *)&k_multi_lean<double, 7>};
    if (na < 2 || na > 7) return nullptr;
    return f64 ? k64[na - 2] : k32[na - 2];
}

// ---------------------------------------------------------------------------
// host: affine forms of postfix programs
// ---------------------------------------------------------------------------
namespace {

struct Form {
    enum Kind { AFFINE, CMP, MAXK, MINK, BAD } kind = BAD;
    double c[KX_MAX_NS + 1] = {};  // c[0] + sum_i c[1 + i] S_i
    double k = 0.0;                // MAXK / MINK: the constant operand
    uint8_t cmp = 0;
    bool constant() const {
        if (kind != AFFINE) return false;
        for (int i = 1; i <= KX_MAX_NS; ++i)
            if (c[i] != 0.0) return false;
        return true;
    }
};

// Evaluates a program symbolically: affine combinations of the spots, a
// comparison of two of them, or max / min of one with a constant (at the
// top only); anything else (averages, dates, products of spots, logic) is BAD.
Form symbolic(const KxProgram &P, int off, int len, int na, bool *neg_top) {
    std::vector<Form> st;
    if (neg_top) *neg_top = false;
    Form bad;
    for (int q = 0; q < len; ++q) {
        const KxIns &I = P.code[off + q];
        const bool last = q == len - 1;
        switch (I.op) {
        case OP_CONST: {
            Form f;
            f.kind = Form::AFFINE;
            f.c[0] = P.cpool[I.arg];
            st.push_back(f);
            break;
        }
        case OP_SPOT: {
            if (I.arg >= na) return bad;
            Form f;
            f.kind = Form::AFFINE;
            f.c[1 + I.arg] = 1.0;
            st.push_back(f);
            break;
        }
        case OP_NEG: {
            if (st.empty()) return bad;
            Form &f = st.back();
            if (f.kind == Form::AFFINE) {
                for (double &x : f.c) x = -x;
            } else if (last && neg_top && (f.kind == Form::MAXK || f.kind == Form::MINK)) {
                *neg_top = true;  // the flow's sign, kept apart (as the lowering emits it)
            } else {
                return bad;
            }
            break;
        }
        case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV:
        case OP_MAX: case OP_MIN:
        case OP_GE: case OP_GT: case OP_LE: case OP_LT: {
            if (st.size() < 2) return bad;
            Form b = st.back();
            st.pop_back();
            Form a = st.back();
            st.pop_back();
            if (a.kind != Form::AFFINE || b.kind != Form::AFFINE) return bad;
            Form r;
            r.kind = Form::AFFINE;
            if (I.op == OP_ADD || I.op == OP_SUB) {
                const double s = I.op == OP_ADD ? 1.0 : -1.0;
                for (int i = 0; i <= KX_MAX_NS; ++i) r.c[i] = a.c[i] + s * b.c[i];
            } else if (I.op == OP_MUL) {
                if (b.constant()) for (int i = 0; i <= KX_MAX_NS; ++i) r.c[i] = a.c[i] * b.c[0];
                else if (a.constant()) for (int i = 0; i <= KX_MAX_NS; ++i) r.c[i] = b.c[i] * a.c[0];
                else return bad;
            } else if (I.op == OP_DIV) {
                if (!b.constant() || b.c[0] == 0.0) return bad;
                for (int i = 0; i <= KX_MAX_NS; ++i) r.c[i] = a.c[i] / b.c[0];
            } else if (I.op == OP_MAX || I.op == OP_MIN) {
                if (!last && !(q == len - 2 && P.code[off + len - 1].op == OP_NEG)) return bad;
                const Form &x = b.constant() ? a : b;
                const Form &kf = b.constant() ? b : a;
                if (!kf.constant()) return bad;
                r = x;
                r.kind = I.op == OP_MAX ? Form::MAXK : Form::MINK;
                r.k = kf.c[0];
            } else {  // comparison: a - b cmp 0
                if (!last) return bad;
                for (int i = 0; i <= KX_MAX_NS; ++i) r.c[i] = a.c[i] - b.c[i];
                r.kind = Form::CMP;
                r.cmp = I.op == OP_GE ? CMP_GE : I.op == OP_GT ? CMP_GT : I.op == OP_LE ? CMP_LE : CMP_LT;
            }
            st.push_back(r);
            break;
        }
        default: return bad;
        }
    }
    if (st.size() != 1) return bad;
    for (double x : st[0].c)
        if (!std::isfinite(x)) return bad;
    if (!std::isfinite(st[0].k)) return bad;
    return st[0];
}

void put_row(const Form &f, int na, double (&c)[KX_MAX_NS + 1], float (&cf)[KX_MAX_NS + 1]) {
    for (int i = 0; i <= na; ++i) {
        c[i] = f.c[i];
        cf[i] = (float)f.c[i];
    }
}

}  // namespace

// The launch arguments of a job, or false when the contract is outside this
// kernel's family (the general kernel then prices it).
static bool multi_lean_args(const Job &j, MultiLeanArgs &A) {
    const KxProgram &P = j.prog;
    const int na = j.dev.n_assets;
    if (na < 2 || na > 7 || P.n_acc || P.err_capable) return false;
    const StaticSchedule S = static_schedule(P, j.tab);
    if (!S.static_ok) return false;
    memset(&A, 0, sizeof A);
    // flows, in slot order
    int fidx[KX_MAX_LEAF];
    int nf = 0;
    std::vector<const StaticSchedule::Flow *> byleaf(P.n_leaf, nullptr);
    for (auto &f : S.flows) byleaf[f.leaf] = &f;
    for (int q = 0; q < P.n_leaf; ++q) {
        fidx[q] = -1;
        if (!byleaf[q]) continue;
        if (nf >= ML_MAXF) return false;
        const KxLeaf &F = P.leaf[q];
        const int f = nf++;
        fidx[q] = f;
        A.all_flows |= 1u << f;
        if (F.kind == AK_CONST) {
            A.f_form[f] = MF_CONST;
            A.f_k[f] = F.sign;
            continue;
        }
        bool neg = false;
        const Form fm = symbolic(P, F.code_off, F.code_len, na, &neg);
        if (fm.kind == Form::AFFINE) {
            A.f_form[f] = MF_AFFINE;
        } else if (fm.kind == Form::MAXK || fm.kind == Form::MINK) {
            A.f_form[f] = fm.kind == Form::MAXK ? MF_MAX : MF_MIN;
            A.f_k[f] = fm.k;
            A.f_kf[f] = (float)fm.k;
        } else {
            return false;
        }
        A.f_sign[f] = neg ? -1.0 : 1.0;
        if (neg) A.f_neg |= (uint8_t)(1u << f);
        put_row(fm, na, A.f_c[f], A.f_cf[f]);
    }
    // barriers: untils on prices that are armed and drop some flow
    std::map<int, std::pair<uint32_t, uint32_t>> at;  // step -> (armed barriers, paid flows)
    for (auto &f : S.flows) at[f.step].second |= 1u << fidx[f.leaf];
    int nb = 0;
    for (int i = 0; i < P.n_trig; ++i) {
        const KxTrig &T = P.trig[i];
        if (T.cond_kind == CK_TIME) continue;
        if (T.kind != TK_UNTIL) return false;
        uint32_t kill = 0;
        for (auto &f : S.flows)
            if ((f.price_untils >> i) & 1u) kill |= 1u << fidx[f.leaf];
        if (S.arm[i] == StaticSchedule::NEVER || kill == 0u) continue;
        const Form fm = symbolic(P, T.code_off, T.code_len, na, nullptr);
        if (fm.kind != Form::CMP || nb >= ML_MAXB) return false;
        const int b = nb++;
        A.kill[b] = (uint8_t)kill;
        A.b_cmp[b] = fm.cmp;
        put_row(fm, na, A.b_c[b], A.b_cf[b]);
        at[S.arm[i]].first |= 1u << b;
    }
    if (at.size() > (size_t)ML_MAXEV) return false;
    for (auto &kv : at) {
        A.ev_step[A.n_ev] = kv.first;
        A.ev_arm[A.n_ev] = (uint8_t)kv.second.first;
        A.ev_pay[A.n_ev] = (uint8_t)kv.second.second;
        ++A.n_ev;
    }
    const ContractDev &d = j.dev;
    A.n_paths = d.n_paths;
    A.path_base = j.path_base;
    A.stream = d.stream;
    A.n_times = d.n_times;
    A.uniform = d.uniform;
    A.uc0 = d.uc0;
    A.uc1 = d.uc1;
    A.uc0f = d.uc0f;
    A.uc1f = d.uc1f;
    const PhiloxKeys K = philox_keys(d.seed);
    memcpy(A.rk, K.rk, sizeof A.rk);
    for (int i = 0; i < KX_MAX_NS; ++i) {
        A.s0[i] = d.s0[i];
        A.drift[i] = d.drift[i];
        A.sigma[i] = d.sigma[i];
        A.s0f[i] = d.s0f[i];
        A.driftf[i] = d.driftf[i];
        A.sigmaf[i] = d.sigmaf[i];
    }
    memcpy(A.chol, d.chol, sizeof A.chol);
    memcpy(A.cholf, d.cholf, sizeof A.cholf);
    return true;
}

bool multi_lean_run(Ctx &c, Job &j, const kx_mc_config &cfg) {
    const char *env = getenv("KX_PATH_KERNEL");
    if (env && strcmp(env, "general") == 0) return false;
    if (j.model.kind != KX_MODEL_MULTI_GBM || cfg.rng == KX_RNG_SHARED_DRAWS) return false;
    MultiLeanArgs A;
    if (!multi_lean_args(j, A)) return false;
    const bool f64 = cfg.precision == KX_PREC_FP64;
    const void *kfn = multi_lean_kernel(f64, j.dev.n_assets);
    if (!kfn) return false;
    const uint64_t n = j.dev.n_paths;
    const int nt = j.dev.n_times;
    c.last.path_steps += n * (uint64_t)(nt > 0 ? nt - 1 : 0);
    j.dev.pv_off = 0;
    if (n == 0) return true;
    std::vector<unsigned char> steps;
    if (f64) pack_steps<double>(j.tab, steps);
    else pack_steps<float>(j.tab, steps);
    c.steps.ensure(steps.size());
    c.disc.ensure(j.tab.disc.size() * sizeof(double));
    c.counters.ensure(64);
    c.pv.ensure(n * sizeof(double));
    KX_CUDA(cudaMemcpyAsync(c.steps.p, steps.data(), steps.size(), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemcpyAsync(c.disc.p, j.tab.disc.data(), j.tab.disc.size() * sizeof(double), cudaMemcpyHostToDevice,
                            c.stream));
    KX_CUDA(cudaMemsetAsync(c.counters.p, 0, 64, c.stream));
    c.last.h2d_bytes += steps.size() + j.tab.disc.size() * sizeof(double) + sizeof A;
    A.steps = c.steps.p;
    A.disc = c.disc.as<double>();
    A.pv = c.pv.as<double>();
    A.next = c.counters.as<unsigned long long>();
    A.steps_done = c.counters.as<unsigned long long>() + 1;
    const int full = persistent_blocks(kfn, ML_BLOCK, 0);
    const uint64_t chunks = (n + ML_CHUNK - 1) / ML_CHUNK;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)full, (chunks + 3) / 4));
    void *args[] = {&A};
    KX_CUDA(cudaEventRecord(c.ev0, c.stream));
    KX_CUDA(cudaLaunchKernel(kfn, dim3(grid), dim3(ML_BLOCK), args, 0, c.stream));
    KX_CUDA(cudaEventRecord(c.ev1, c.stream));
    c.last.kernel_launches++;
    c.last.grid_blocks = (uint32_t)grid;
    c.last.block_threads = (uint32_t)ML_BLOCK;
    c.last.path_kernel = 5u;
    unsigned long long hc[2] = {0, 0};
    KX_CUDA(cudaMemcpyAsync(hc, c.counters.p, sizeof hc, cudaMemcpyDeviceToHost, c.stream));
    KX_CUDA(cudaStreamSynchronize(c.stream));
    float ms = 0.f;
    KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.last.kernel_ms += ms;
    c.last.steps_simulated += hc[1];
    return true;
}

}  // namespace kx
