// paths_lean.cuh — the path kernel for barrier contracts (k_lean).
//
// Same job as k_paths (simulate, evaluate the contract, write one value per
// path) for the contracts whose price-dependent conditions are all
// `Spot cmp Const` and which keep no running averages or extrema: European
// and Bermudan payoffs, single and double barriers (knock-out and knock-in),
// first-touch and digital contracts, scaled flows. The per-step work of such
// a contract reduces to one test: the log-spot left the open interval
// (lo, hi) of the live barriers, or the step reached the next step at which
// a time condition can change. A lane runs its path without looking at the
// contract until that test fires; the event itself (firing cascade, flows,
// knock-out) is the general handler `on_event` of k_paths, so both kernels
// give the same value for every path.
//
// Lanes are not step-synchronous: each lane draws the Philox block of its
// own next step (4 GBM steps or 2 Heston steps per 128-bit draw) and may
// stop inside it at an event; after the event it resumes from the same block
// with the used normals skipped. Idle lanes take new paths at the top of the
// next block, as in k_paths; step 0 of a new path is its first event, so the
// kernel has a single call site of the out-of-line handler. Lanes with an
// event wait for one another (GBM) so that one handler round serves several.
#pragma once
#include "paths_kernel.cuh"

namespace kx {

// Interval test of the live barrier slots: an up slot (>=, >) fires when
// y >= hi, a down slot (<=, <) when y <= lo. Strict comparisons use the next
// representable threshold, which gives the same decision for finite y.
template <class Real>
__device__ __forceinline__ void lean_window(const KxProgram &P, const Real *thr, uint32_t live, Real &hi, Real &lo) {
    hi = Real(INFINITY);
    lo = Real(-INFINITY);
    uint32_t m = live & P.price_mask;
    while (m) {
        const int i = __ffs(m) - 1;
        m &= m - 1;
        const KxTrig &T = P.trig[i];
        const Real t = thr[T.spot_slot];
        switch (T.cmp) {
        case CMP_GE: hi = fmin(hi, t); break;
        case CMP_GT: hi = fmin(hi, next_up(t)); break;
        case CMP_LE: lo = fmax(lo, t); break;
        default: lo = fmax(lo, next_down(t)); break;
        }
    }
}

// Everything the contract does at step k for a lane whose test fired (or at
// t = 0). Returns the new state; st.done is set when no flow can change.
template <class Real>
__device__ __forceinline__ Trig lean_event(const KxProgram *Pp, const ContractDev *Cp, const StepRec<Real> *R,
                                           const Real *thr, const double *D, Real s0, Real y, int k, Trig st) {
    const KxProgram &P = *Pp;
    const uint32_t live = st.armed & ~st.resolved;
    uint32_t bits = 0;
    uint32_t m = live & P.price_mask;
    while (m) {
        const int i = __ffs(m) - 1;
        m &= m - 1;
        const KxTrig &T = P.trig[i];
        if (cmp_y<Real>(T.cmp, y, thr[T.spot_slot])) bits |= 1u << i;
    }
    if (k >= st.nte) bits |= live & P.time_mask & R[k].tt;
    if (k > 0) {
        if (!bits) return st;
        if ((bits & ~P.until_mask) == 0u) {  // knock-out only: drop the flows below, nothing is acquired
            st.resolved |= bits;
            uint32_t u = bits;
            while (u) {
                const int i = __ffs(u) - 1;
                u &= u - 1;
                st.dead |= P.trig[i].leaves & ~st.emitted;
            }
            st.done = !P.err_capable && (P.all_leaves & ~(st.emitted | st.dead)) == 0u;
            return st;
        }
    } else if (!bits && !P.root_leaves) {  // nothing happens at t = 0
        st.nte = P.init_nte;
        return st;
    }
    // Inline when the firing arms nothing new and every acquired flow has a
    // constant or closed-form amount: on_event's steps in on_event's order
    // (knock-outs first, then the flows in slot order, then the next time
    // event), so the value is the same.
    uint32_t arm = 0, acq = k == 0 ? P.root_leaves : 0u;
    uint32_t w = bits & P.when_mask;
    while (w) {
        const int i = __ffs(w) - 1;
        w &= w - 1;
        arm |= P.trig[i].fire_arm;
        acq |= P.trig[i].leaves;
    }
    acq &= ~st.emitted;
    if ((arm & ~st.armed) == 0u && !P.err_capable && (acq & ~P.simple_leaves) == 0u) {
        st.resolved |= bits;
        uint32_t u = bits & P.until_mask;
        while (u) {
            const int i = __ffs(u) - 1;
            u &= u - 1;
            st.dead |= P.trig[i].leaves & ~st.emitted;
        }
        acq &= ~st.dead;
        if (acq) {
            const Real S = spot_of<Real>(s0, y);
            while (acq) {
                const int j = __ffs(acq) - 1;
                acq &= acq - 1;
                const KxLeaf &F = P.leaf[j];
                const double amt = F.kind == AK_CONST ? F.sign : (double)fast_amount<Real>(P, F, S);
                st.pv = __dadd_rn(st.pv, __dmul_rn(amt, D[k]));
                st.emitted |= 1u << j;
            }
        }
        const uint32_t live_t = st.armed & ~st.resolved & P.time_mask;
        int nte = INT_MAX;
        if (live_t & ~P.mono_mask) {
            nte = k + 1;
        } else {
            uint32_t t = live_t;
            while (t) {
                const int i = __ffs(t) - 1;
                t &= t - 1;
                nte = min(nte, P.first_true[i]);
            }
        }
        st.nte = nte;
        st.done = (P.all_leaves & ~(st.emitted | st.dead)) == 0u;
        return st;
    }
    return on_event<Real>(Pp, Cp, R, thr, D, nullptr, nullptr, KX_BLOCK, s0, y, k, bits, 0u, 0, st, nullptr);
}

// ---------------------------------------------------------------------------
// Static schedules. When every when/anytime condition of a contract reads
// only the time, every until reads either the time or Spot-cmp-Const, and
// every flow amount is constant or closed-form, the whole contract is a
// fixed list of steps at which barriers are armed and flows are paid, plus
// the barrier knock-outs of each path. The host compiles that list
// (StaticDev) and the kernel keeps only a few masks per path: the live
// barriers, the flows still to pay, the next event and the value.
// Flows are numbered by their flow slot, so the value adds them in the same
// order as on_event and is the same bit for bit.
// ---------------------------------------------------------------------------
constexpr int KX_MAX_SEV = 64;
constexpr int KX_MAX_SM = 2;  // smoothed barriers a static schedule carries in registers

struct StaticDev {
    int32_t n_ev;
    uint32_t up_mask;    // barrier slots that fire upwards (y >= thr); the others downwards (y <= thr)
    uint32_t all_flows;  // flow slots of the schedule (flows knocked by time-only untils are left out)
    uint32_t gen_flows;  // flow slots whose amount reads the accumulator: evaluated by the interpreter
    int32_t acc_on;      // the contract keeps one accumulator of the spot (slot 0): average, max or min
    int32_t acc_from;    // its window: steps acc_from .. acc_to
    int32_t acc_to;
    int32_t acc_kind;    // KxAccKind
    int32_t ev_step[KX_MAX_SEV];
    uint32_t ev_arm[KX_MAX_SEV];  // barrier slots armed at that step (tested at once)
    uint32_t ev_pay[KX_MAX_SEV];  // flow slots paid at that step unless knocked out
    uint32_t kill[KX_MAX_TRIG];   // flow slots dropped when barrier slot i knocks
    float thr32[KX_MAX_TRIG];     // log-spot thresholds, strict comparisons made inclusive
    double thr64[KX_MAX_TRIG];
    uint8_t f_fast[KX_MAX_LEAF];  // KxFastAmount of the flow slot (FA_NONE: constant amount)
    double f_k[KX_MAX_LEAF];      // its constant K
    double f_sign[KX_MAX_LEAF];   // its sign (the constant amount itself for FA_NONE)
    uint32_t f_neg;               // flow slots whose sign is negative (tested without FP64)
    // Smoothed barriers (a bump of the smoothed payoff): until(Spot cmp Const)
    // slots that never knock; from their arming step on, every step multiplies
    // the slot's weight by smooth_weight(x), x = (y - thr) * mul (mul = +-1/w,
    // negative for a downward barrier), and a paid flow is multiplied by the
    // weights of the slots above it, in slot order (on_event's arithmetic).
    int32_t n_sm;
    int32_t sm_arm[KX_MAX_SM];     // first weighed step
    uint32_t sm_flows[KX_MAX_SM];  // flow slots under the barrier
    float sm_thr32[KX_MAX_SM], sm_mul32[KX_MAX_SM];
    double sm_thr64[KX_MAX_SM], sm_mul64[KX_MAX_SM];
};

struct SLane {
    uint32_t live;  // armed barriers not knocked out
    uint32_t rem;   // flows neither paid nor dropped
    int e;          // next static event
    double pv;
};

template <class Real>
__device__ __forceinline__ Real sthr(const StaticDev &T, int i) {
    return sizeof(Real) == 4 ? (Real)T.thr32[i] : (Real)T.thr64[i];
}

// One spot added to the accumulator, as the general kernel adds it
// (contract_step): a running max or min, or the sum of an average,
// compensated (Kahan) in FP32 and plain in FP64. AK: the kind (KxAccKind)
// when known at compile time, -1 to read `kind`.
template <class Real, int AK = -1>
__device__ __forceinline__ void acc_add(int kind, Real &v, Real &c, Real x) {
    if (AK >= 0) kind = AK;
    if (kind == ACC_MAX) {
        v = fmax(v, x);
    } else if (kind == ACC_MIN) {
        v = fmin(v, x);
    } else if (sizeof(Real) == 8) {
        v = v + x;
    } else {
        const Real yk = x - c;
        const Real t = v + yk;
        c = (t - v) - yk;
        v = t;
    }
}

// The contract at step k of a static-schedule path: knock-outs of the live
// barriers, then the static event of step k (barriers armed and tested at
// once, flows paid), as on_event orders them (pricer.rs:374-433). ACC: flows
// in gen_flows read the running average (av, ac: its sum and compensation),
// evaluated by the interpreter as on_event evaluates them.
// Smoothed barriers of one contract (warp-uniform, from StaticDev) and the
// weight update of one step: slot q (live in `sml`, armed at or before step
// k) multiplies its weight by smooth_weight((y - t_q) m_q), skipping the
// steps where that weight is exactly 1.
template <class Real>
struct SmoothPar {
    int n;
    int a0, a1;
    Real t0, t1, m0, m1;
};

template <class Real>
__device__ __forceinline__ SmoothPar<Real> smooth_par(const StaticDev &T) {
    const bool f = sizeof(Real) == 4;
    return SmoothPar<Real>{T.n_sm, T.sm_arm[0], T.sm_arm[1],
                           f ? (Real)T.sm_thr32[0] : (Real)T.sm_thr64[0], f ? (Real)T.sm_thr32[1] : (Real)T.sm_thr64[1],
                           f ? (Real)T.sm_mul32[0] : (Real)T.sm_mul64[0], f ? (Real)T.sm_mul32[1] : (Real)T.sm_mul64[1]};
}

template <class Real>
__device__ __forceinline__ void smooth_step(const SmoothPar<Real> &sp, Real y, int k, uint32_t sml, Real &w0,
                                            Real &w1) {
    if ((sml & 1u) && k >= sp.a0) {
        const Real x = (y - sp.t0) * sp.m0;
        if (x > smooth_cut<Real>()) w0 *= logistic(x);
    }
    if ((sml & 2u) && k >= sp.a1) {
        const Real x = (y - sp.t1) * sp.m1;
        if (x > smooth_cut<Real>()) w1 *= logistic(x);
    }
}

// A live smoothed weight reached exactly 0: its flows can add nothing more.
template <class Real>
__device__ __forceinline__ bool smooth_zero(uint32_t sml, Real w0, Real w1) {
    return ((sml & 1u) && w0 == Real(0)) || ((sml & 2u) && w1 == Real(0));
}

template <class Real, bool ACC = false, bool SM = false>
__device__ __forceinline__ void static_event(const StaticDev &T, const double *D, Real s0, Real y, int k, SLane &L,
                                             const KxProgram *P = nullptr, Real av = Real(0), Real ac = Real(0),
                                             Real w0 = Real(1), Real w1 = Real(1), uint32_t *sml = nullptr) {
    uint32_t m = L.live;
    while (m) {
        const int i = __ffs(m) - 1;
        m &= m - 1;
        const Real t = sthr<Real>(T, i);
        if ((T.up_mask >> i) & 1u ? y >= t : y <= t) {
            L.live &= ~(1u << i);
            L.rem &= ~T.kill[i];
        }
    }
    if (L.e < T.n_ev && T.ev_step[L.e] == k) {
        uint32_t a = T.ev_arm[L.e];
        while (a) {
            const int i = __ffs(a) - 1;
            a &= a - 1;
            const Real t = sthr<Real>(T, i);
            if ((T.up_mask >> i) & 1u ? y >= t : y <= t) L.rem &= ~T.kill[i];
            else L.live |= 1u << i;
        }
        uint32_t pay = T.ev_pay[L.e] & L.rem;
        if (pay) {
            const Real S = spot_of<Real>(s0, y);
            while (pay) {
                const int j = __ffs(pay) - 1;
                pay &= pay - 1;
                double amt = T.f_sign[j];
                if (ACC && ((T.gen_flows >> j) & 1u)) {
                    Real accbuf[2] = {av, ac};
                    uint32_t e = 0;
                    amt = (double)eval_code<Real>(*P, P->leaf[j].code_off, P->leaf[j].code_len,
                                                  AccView<Real>{accbuf, 1}, 0u, k, S, e);
                } else if (T.f_fast[j] != FA_NONE) {
                    const Real K = (Real)T.f_k[j];
                    Real r;
                    switch (T.f_fast[j]) {
                    case FA_CALL: r = fmax(S - K, Real(0)); break;
                    case FA_PUT: r = fmax(K - S, Real(0)); break;
                    case FA_SPOT: r = S; break;
                    default: r = K; break;
                    }
                    amt = (double)(((T.f_neg >> j) & 1u) ? -r : r);
                }
                if (SM) {  // the weights of the smoothed barriers above the flow, in slot order
                    if (T.n_sm > 0 && ((T.sm_flows[0] >> j) & 1u) && k >= T.sm_arm[0]) amt *= (double)w0;
                    if (T.n_sm > 1 && ((T.sm_flows[1] >> j) & 1u) && k >= T.sm_arm[1]) amt *= (double)w1;
                }
                L.pv = __dadd_rn(L.pv, __dmul_rn(amt, D[k]));
            }
        }
        L.rem &= ~T.ev_pay[L.e];
        ++L.e;
    }
    if (SM) {  // a weight that reached 0 zeroes its flows: drop them (they would add +-0)
        if ((*sml & 1u) && w0 == Real(0)) {
            L.rem &= ~T.sm_flows[0];
            *sml &= ~1u;
        }
        if ((*sml & 2u) && w1 == Real(0)) {
            L.rem &= ~T.sm_flows[1];
            *sml &= ~2u;
        }
    }
}

template <class Real>
__device__ __forceinline__ void static_window(const StaticDev &T, uint32_t live, Real &hi, Real &lo) {
    hi = Real(INFINITY);
    lo = Real(-INFINITY);
    uint32_t m = live;
    while (m) {
        const int i = __ffs(m) - 1;
        m &= m - 1;
        const Real t = sthr<Real>(T, i);
        if ((T.up_mask >> i) & 1u) hi = fmin(hi, t);
        else lo = fmax(lo, t);
    }
}

template <class Real>
struct HestonPar {
    Real r, kappa, theta, sigma_v, rho, rho_perp;
    int scheme;
};

// Grid steps per Philox block (four normals) and normals per grid step of a
// path model. The _PAIR models are the coarse paths of multilevel pairs: a
// coarse GBM step adds the normals of its two fine steps (simulator.rs:373-377),
// a coarse Heston step sums the two fine (z1, z2) pairs over sqrt 2 (:656-661).
template <int MODEL>
constexpr int lean_spb() { return MODEL == M_GBM ? 4 : MODEL == M_HESTON_PAIR ? 1 : 2; }
template <int MODEL>
constexpr int lean_draws() { return MODEL == M_GBM ? 1 : MODEL == M_HESTON_PAIR ? 4 : 2; }
template <int MODEL>
constexpr bool lean_gbmlike() { return MODEL == M_GBM || MODEL == M_GBM_PAIR; }

// Grid step j of a Philox block, as k_paths steps it.
template <class Real, int MODEL>
__device__ __forceinline__ void lean_model_step(const HestonPar<Real> &hp, Real c0, Real c1, const Real (&zz)[4], int j,
                                                Real &y, Real &v) {
    if (MODEL == M_GBM) {
        y = gbm_step(y, c0, c1, zz[j]);  // log-space exact GBM step (simulator.rs:238-245)
    } else if (MODEL == M_GBM_PAIR) {
        y = gbm_step(y, c0, c1, zz[2 * j] + zz[2 * j + 1]);
    } else if (MODEL == M_HESTON) {
        heston_step<Real>(hp.r, hp.kappa, hp.theta, hp.sigma_v, hp.rho, hp.rho_perp, hp.scheme, c0, c1, zz[2 * j],
                          zz[2 * j + 1], y, v);
    } else {
        const Real inv_sqrt2 = Real(0.70710678118654752440);
        heston_step<Real>(hp.r, hp.kappa, hp.theta, hp.sigma_v, hp.rho, hp.rho_perp, hp.scheme, c0, c1,
                          (zz[0] + zz[2]) * inv_sqrt2, (zz[1] + zz[3]) * inv_sqrt2, y, v);
    }
}

// The steps of one Philox block from offset `off` on, up to the first step at
// which the barrier window or the step limit fires (returns true; k is that
// step) or to the end of the block (k is the next step). UNI: every step has
// the coefficients (uc0, uc1), so the step table is not read. The states are
// the same bit for bit whichever way the block is walked. ACC: the spot of
// every step in af .. at is added to the accumulator of kind AK (av, ac;
// AK < 0: none).
template <class Real, int MODEL, bool UNI, int AK, bool SM = false>
__device__ __forceinline__ bool lean_steps(const StepRec<Real> *R, Real uc0, Real uc1, const HestonPar<Real> &hp,
                                           const Real (&zz)[4], int off, Real hi, Real lo, int lim, Real &y, Real &v,
                                           int &k, Real s0, int af, int at, Real &av, Real &ac,
                                           const SmoothPar<Real> *sp = nullptr, uint32_t sml = 0u,
                                           Real *w0 = nullptr, Real *w1 = nullptr) {
    constexpr bool ACC = AK >= 0;
    constexpr int SPB = lean_spb<MODEL>();
    // GBM: a whole block is stepped first and tested once (min and max of its
    // states against the window, its last step against the limit); only a
    // block in which something fires is walked again step by step. A Heston
    // step is long enough that redoing it costs more than the test saves.
    if (lean_gbmlike<MODEL>() && off == 0) {
        Real yy = y, vv = v, mx = Real(-INFINITY), mn = Real(INFINITY);
        Real av2 = av, ac2 = ac;
        Real w0c = SM ? *w0 : Real(1), w1c = SM ? *w1 : Real(1);
#pragma unroll
        for (int j = 0; j < SPB; ++j) {
            Real c0 = uc0, c1 = uc1;
            if (!UNI) {
                const StepRec<Real> rec = R[min(k + j, lim)];
                c0 = rec.c0;
                c1 = rec.c1;
            }
            lean_model_step<Real, MODEL>(hp, c0, c1, zz, j, yy, vv);
            if (ACC && k + j >= af && k + j <= at) acc_add<Real, AK>(AK, av2, ac2, spot_of<Real>(s0, yy));
            if (SM) smooth_step<Real>(*sp, yy, k + j, sml, w0c, w1c);
            mx = fmax(mx, yy);
            mn = fmin(mn, yy);
        }
        if (mx < hi && mn > lo && k + SPB - 1 < lim && !(SM && smooth_zero<Real>(sml, w0c, w1c))) {
            // nothing fires inside the block
            y = yy;
            v = vv;
            if (ACC) {
                av = av2;
                ac = ac2;
            }
            if (SM) {
                *w0 = w0c;
                *w1 = w1c;
            }
            k += SPB;
            return false;
        }
    }
    bool ev = false;  // step by step up to the event
#pragma unroll
    for (int j = 0; j < SPB; ++j) {
        if (j >= off && !ev) {
            Real c0 = uc0, c1 = uc1;
            if (!UNI) {
                const StepRec<Real> rec = R[k];
                c0 = rec.c0;
                c1 = rec.c1;
            }
            lean_model_step<Real, MODEL>(hp, c0, c1, zz, j, y, v);
            if (ACC && k >= af && k <= at) acc_add<Real, AK>(AK, av, ac, spot_of<Real>(s0, y));
            if (SM) smooth_step<Real>(*sp, y, k, sml, *w0, *w1);
            if (y >= hi || y <= lo || k >= lim || (SM && smooth_zero<Real>(sml, *w0, *w1))) ev = true;
            else ++k;
        }
    }
    return ev;
}

// ACC (static schedules only): the contracts may keep one accumulator of the
// spot (slot 0: an average, a running max or min), in registers. SM (static
// schedules only, no accumulator): the contracts' barriers are smoothed
// (survival weights in registers instead of knock-outs).
template <class Real, int MODEL, int MINB, bool STATIC, bool ACC = false, bool SM = false>
__global__ void __launch_bounds__(KX_BLOCK, MINB) k_lean(const PathArgs A) {
    static_assert(!ACC || STATIC, "averages need a static schedule");
    static_assert(!SM || (STATIC && !ACC), "smoothed barriers need a static schedule without an accumulator");
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    constexpr int SPB = lean_spb<MODEL>();  // grid steps per Philox block
    constexpr int DRAWS = lean_draws<MODEL>();
    constexpr bool GBMLIKE = lean_gbmlike<MODEL>();
    constexpr bool HESTON = !GBMLIKE;
    // Event batching: a lane whose path reached an event waits (up to
    // EV_WAIT blocks) until EV_BATCH lanes of its warp have one, so the
    // handler runs once for many lanes instead of once per lane. Worth it
    // for GBM, whose blocks are short next to the handler; a Heston block is
    // long enough that waiting costs more than it saves.
    // (GBM: batches of 6 with waits of 3 rounds of 8 blocks took 1.341 ms on
    // the 4M-path up-and-out call, 8 / 4 rounds of 4 blocks 1.362 ms.)
    constexpr int EV_BATCH = GBMLIKE ? 6 : 1;
    constexpr int EV_WAIT = GBMLIKE ? 3 : 8;  // rounds of BPI blocks
    // Philox blocks a lane steps through per round of the warp loop: eight for
    // GBM (32 steps) cut the per-round hand-out and event ballots per step.
    constexpr int BPI = GBMLIKE ? 8 : 1;

    // warp-uniform work state (path indices are per contract, < 2^32)
    int cur = -1, pend = -1;
    uint32_t nx = 0, end = 0;
    bool drained = false;
    const KxProgram *P = nullptr;
    const ContractDev *C = nullptr;
    const StepRec<Real> *R = nullptr;
    const Real *thr = nullptr;
    const double *D = nullptr;
    uint64_t pv_off = 0, seed = 0;
    uint32_t stream = 0;
    int nt = 0;
    bool uniform = false;
    Real s0 = 1, uc0 = 0, uc1 = 0;
    Real hr = 0, hk = 0, hth = 0, hsv = 0, hrho = 0, hrp = 0, hv0 = 0;
    int scheme = KX_HESTON_REFERENCE_FLOOR;

    // lane state
    bool busy = false;
    uint32_t path = 0;
    int k = 0, lim = 0;
    Real y = 0, v = 0, hi = 0, lo = 0;
    Trig st{0, 0, 0, 0, 0, 0, 0, 0, 0.0};
    SLane sl{0u, 0u, 0, 0.0};
    uint32_t my_steps = 0;
    Real av = 0, ac = 0;      // accumulator: value (sum, max or min) and compensation
    int acc_f = 1, acc_t = 0; // warp-uniform: the contract's accumulator window (empty: none)
    int acc_k = ACC_SUM;      // and its kind
    SmoothPar<Real> sp{0, 0, 0, Real(0), Real(0), Real(0), Real(0)};  // warp-uniform: smoothed barriers
    Real sw0 = 1, sw1 = 1;    // lane: their survival weights
    uint32_t sml = 0u;        // lane: the smoothed barriers whose weight is not yet 0
    bool evp = false;  // this lane waits with an event at step k
    int wait = 0;      // warp-uniform: blocks since the last handler round
    // static schedules: every path of a contract is at S = s0 at t = 0, so its state after
    // step 0 (barriers armed and tested, flows of t = 0 paid, the window, the next event) is
    // the same for all of them: computed once per contract and warp, copied at each hand-out
    // (not in the accumulator and smoothed families, whose registers the copy would strain)
    struct Start0 {
        SLane sl;
        Real hi, lo, av, ac, w0, w1;
        int lim;
        uint32_t sml;
        int done;
    };
    __shared__ Start0 start0[KX_BLOCK / 32];
    Start0 &T0 = start0[threadIdx.x >> 5];
    // a new path on this lane: S = s0, step 0 next
    auto start_path = [&](uint32_t p) {
        path = p;
        busy = true;
        y = Real(0);
        v = fmax(hv0, Real(0));
        // as k_paths starts an accumulator
        av = acc_k == ACC_MAX ? Real(-INFINITY) : acc_k == ACC_MIN ? Real(INFINITY) : Real(0);
        ac = Real(0);
        if (STATIC) {
            sl = SLane{0u, static_cast<const StaticDev *>(A.statics)[cur].all_flows, 0, 0.0};
        } else {
            st = Trig{P->root_arm, 0u, 0u, 0u, 0u, st.err, 0, 0, 0.0};
        }
        if (SM) {
            sw0 = Real(1);
            sw1 = Real(1);
            sml = (1u << sp.n) - 1u;
        }
        k = 0;
    };
    // static schedules: the contract at step k of this lane's path (knock-outs,
    // the static event of step k), then the next event step; the path's value
    // is stored when nothing more can be paid
    auto static_lane_event = [&]() {
        const StaticDev &T = static_cast<const StaticDev *>(A.statics)[cur];
        if (ACC && k == 0 && acc_f <= 0 && 0 <= acc_t)  // the spot at t = 0 (steps >= 1: lean_steps)
            acc_add<Real>(acc_k, av, ac, spot_of<Real>(s0, y));
        if (SM && k == 0) smooth_step<Real>(sp, y, 0, sml, sw0, sw1);  // t = 0 (steps >= 1: lean_steps)
        static_event<Real, ACC, SM>(T, D, s0, y, k, sl, P, av, ac, sw0, sw1, &sml);
        static_window<Real>(T, sl.live, hi, lo);
        lim = sl.e < T.n_ev ? min(T.ev_step[sl.e], nt - 1) : nt - 1;
        ++k;
        if (sl.rem == 0u || k >= nt) {
            A.pv[pv_off + path] = sl.pv;
            busy = false;
        }
    };

    while (true) {
        // ---- hand paths to idle lanes (warp-uniform control) ----
        unsigned idle = __ballot_sync(FULL, !busy);
        while (idle) {
            if (nx >= end) {
                int it = pend;
                if (it < 0) {
                    if (drained) break;
                    if (lane == 0) it = (int)atomicAdd(A.item_counter, 1u);
                    it = __shfl_sync(FULL, it, 0);
                    if (it >= (int)A.n_items) {
                        drained = true;
                        break;
                    }
                }
                const WorkItem w = fetch_item(A, it);
                if (w.contract != cur) {
                    if (cur >= 0 && idle != FULL) {  // finish the current contract first
                        pend = it;
                        break;
                    }
                    cur = w.contract;
                    C = A.cons + cur;
                    P = A.progs + C->prog;
                    R = reinterpret_cast<const StepRec<Real> *>(A.steps) + C->step_off;
                    thr = reinterpret_cast<const Real *>(A.thr) + (size_t)cur * KX_MAX_NS * KX_MAX_SPOT;
                    D = A.disc + C->disc_off;
                    pv_off = C->pv_off;
                    seed = C->seed;
                    stream = C->stream;
                    nt = C->n_times;
                    uniform = C->uniform != 0;
                    s0 = pick<Real>(C->s0[0], C->s0f[0]);
                    uc0 = pick<Real>(C->uc0, C->uc0f);
                    uc1 = pick<Real>(C->uc1, C->uc1f);
                    if (HESTON) {
                        hr = pick<Real>(C->r, C->rf);
                        hk = pick<Real>(C->kappa, C->kappaf);
                        hth = pick<Real>(C->theta, C->thetaf);
                        hsv = pick<Real>(C->sigma_v, C->sigma_vf);
                        hrho = pick<Real>(C->rho, C->rhof);
                        hrp = pick<Real>(C->rho_perp, C->rho_perpf);
                        hv0 = pick<Real>(C->v0, C->v0f);
                        scheme = C->heston_scheme;
                    }
                    if (ACC) {
                        const StaticDev &T = static_cast<const StaticDev *>(A.statics)[cur];
                        acc_f = T.acc_on ? T.acc_from : 1;
                        acc_t = T.acc_on ? T.acc_to : 0;
                        acc_k = T.acc_kind;
                    }
                    if (SM) sp = smooth_par<Real>(static_cast<const StaticDev *>(A.statics)[cur]);
                    if (STATIC && !ACC && !SM) {  // every lane is idle here: the warp computes the contract's step 0
                        const StaticDev &T = static_cast<const StaticDev *>(A.statics)[cur];
                        SLane t{0u, T.all_flows, 0, 0.0};
                        Real tav = acc_k == ACC_MAX ? Real(-INFINITY) : acc_k == ACC_MIN ? Real(INFINITY) : Real(0);
                        Real tac = Real(0), tw0 = Real(1), tw1 = Real(1);
                        uint32_t tsml = SM ? (1u << sp.n) - 1u : 0u;
                        if (ACC && acc_f <= 0 && 0 <= acc_t) acc_add<Real>(acc_k, tav, tac, spot_of<Real>(s0, Real(0)));
                        if (SM) smooth_step<Real>(sp, Real(0), 0, tsml, tw0, tw1);
                        static_event<Real, ACC, SM>(T, D, s0, Real(0), 0, t, P, tav, tac, tw0, tw1, &tsml);
                        Real thi, tlo;
                        static_window<Real>(T, t.live, thi, tlo);
                        const int tlim = t.e < T.n_ev ? min(T.ev_step[t.e], nt - 1) : nt - 1;
                        if (lane == 0)
                            T0 = Start0{t, thi, tlo, tav, tac, tw0, tw1, tlim, tsml, (t.rem == 0u || nt <= 1) ? 1 : 0};
                        __syncwarp();
                    }
                }
                pend = -1;
                nx = (uint32_t)w.first;
                end = (uint32_t)(w.first + w.count);
                continue;
            }
            const int nidle = __popc(idle);
            const uint32_t avail = end - nx;
            const int take = avail < (uint32_t)nidle ? (int)avail : nidle;
            const int rank = __popc(idle & lt);
            if (!busy && rank < take) {
                // new path: the contract at step 0 runs as this lane's first event (for static
                // schedules its outcome is the contract's Start0, copied; the accumulator and
                // smoothed families, tighter on registers, run it; a path that ends at step 0
                // leaves the lane idle)
                if (STATIC && (ACC || SM)) {
                    start_path(nx + (uint32_t)rank);
                    static_lane_event();
                } else if (STATIC) {
                    path = nx + (uint32_t)rank;
                    busy = true;
                    y = Real(0);
                    v = fmax(hv0, Real(0));
                    sl = T0.sl;
                    hi = T0.hi;
                    lo = T0.lo;
                    lim = T0.lim;
                    av = T0.av;
                    ac = T0.ac;
                    if (SM) {
                        sw0 = T0.w0;
                        sw1 = T0.w1;
                        sml = T0.sml;
                    }
                    k = 1;
                    if (T0.done) {
                        A.pv[pv_off + path] = sl.pv;
                        busy = false;
                    }
                } else {
                    start_path(nx + (uint32_t)rank);
                }
            }
            nx += (uint32_t)take;
            if (take == 0) break;
            idle = __ballot_sync(FULL, !busy);
        }
        if (__ballot_sync(FULL, busy) == 0u) {
            if (drained && pend < 0 && nx >= end) break;
            continue;
        }

        // ---- one Philox block of this lane's path, up to the next event ----
        bool ev = busy && (k == 0 || evp);  // a waiting event or step 0 of a new path
        if (busy && !ev) {
            for (int bb = 0; bb < BPI && !ev; ++bb) {
                const uint32_t km1 = (uint32_t)(k - 1);
                const uint32_t blk = km1 / SPB;
                const int off = (int)(km1 % SPB);
                Real zz[4];
                if (A.z64 == nullptr && A.z32 == nullptr) {
                    const uint4 ctr = make_uint4(blk, path, 0u, stream);
                    const uint4 w = A.rk_ok ? philox4x32_10_rk(ctr, A.rk)
                                            : philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
                    box_muller(w.x, w.y, zz[0], zz[1]);
                    box_muller(w.z, w.w, zz[2], zz[3]);
                } else {
                    const uint64_t d0 = (uint64_t)blk * SPB * DRAWS;
                    const uint64_t base = (uint64_t)path * A.z_dpp + d0;
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        zz[j] = d0 + j < A.z_dpp ? (A.z64 ? (Real)A.z64[base + j] : (Real)A.z32[base + j]) : Real(0);
                }
                const int k_in = k;
                const HestonPar<Real> hp{hr, hk, hth, hsv, hrho, hrp, scheme};
                if (SM) {
                    if (uniform)
                        ev = lean_steps<Real, MODEL, true, -1, true>(R, uc0, uc1, hp, zz, off, hi, lo, lim, y, v, k, s0,
                                                                     0, -1, av, ac, &sp, sml, &sw0, &sw1);
                    else
                        ev = lean_steps<Real, MODEL, false, -1, true>(R, uc0, uc1, hp, zz, off, hi, lo, lim, y, v, k,
                                                                      s0, 0, -1, av, ac, &sp, sml, &sw0, &sw1);
                } else if (!ACC) {
                    if (uniform)
                        ev = lean_steps<Real, MODEL, true, -1>(R, uc0, uc1, hp, zz, off, hi, lo, lim, y, v, k, s0, 0, -1,
                                                               av, ac);
                    else
                        ev = lean_steps<Real, MODEL, false, -1>(R, uc0, uc1, hp, zz, off, hi, lo, lim, y, v, k, s0, 0,
                                                                -1, av, ac);
                } else if (acc_k == ACC_SUM) {  // the kind is warp-uniform: one branch per block, none per step
                    if (uniform)
                        ev = lean_steps<Real, MODEL, true, ACC_SUM>(R, uc0, uc1, hp, zz, off, hi, lo, lim, y, v, k, s0,
                                                                    acc_f, acc_t, av, ac);
                    else
                        ev = lean_steps<Real, MODEL, false, ACC_SUM>(R, uc0, uc1, hp, zz, off, hi, lo, lim, y, v, k, s0,
                                                                     acc_f, acc_t, av, ac);
                } else if (acc_k == ACC_MAX) {
                    ev = lean_steps<Real, MODEL, false, ACC_MAX>(R, uc0, uc1, hp, zz, off, hi, lo, lim, y, v, k, s0,
                                                                 acc_f, acc_t, av, ac);
                } else {
                    ev = lean_steps<Real, MODEL, false, ACC_MIN>(R, uc0, uc1, hp, zz, off, hi, lo, lim, y, v, k, s0,
                                                                 acc_f, acc_t, av, ac);
                }
                my_steps += (uint32_t)(k - k_in) + (ev ? 1u : 0u);
            }
        }
        // ---- events: handled together once enough lanes wait for one ----
        evp = ev;
        const unsigned pm = __ballot_sync(FULL, evp);
        if (pm) {
            const unsigned run = __ballot_sync(FULL, busy && !evp);  // lanes still stepping
            const unsigned k0 = __ballot_sync(FULL, evp && k == 0);  // new paths wait for step 0
            ++wait;
            if (__popc(pm) >= EV_BATCH || run == 0u || wait >= EV_WAIT || k0) {
                wait = 0;
                if (evp) {
                    evp = false;
                    if (STATIC) {
                        static_lane_event();
                    } else {
                        st = lean_event<Real>(P, C, R, thr, D, s0, y, k, st);
                        lean_window<Real>(*P, thr, st.armed & ~st.resolved, hi, lo);
                        lim = min(st.nte, nt - 1);
                        ++k;
                        if (st.done != 0 || k >= nt) {
                            A.pv[pv_off + path] = st.pv;
                            busy = false;
                        }
                    }
                }
            }
        }
    }
    // counters: one atomic per warp
    unsigned long long tot = (unsigned long long)my_steps;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
    uint32_t err = st.err;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) err |= __shfl_xor_sync(FULL, err, o);
    if (lane == 0) {
        if (tot) atomicAdd(A.steps_done, tot);
        if (err) atomicOr(A.err_word, err);
    }
}

// which: fp64 0/1; returns nullptr for a missing register budget.
// acc: the static family with a running average (stat must be set).
const void *lean_kernel_gbm(int fp64, int minb, bool stat, bool acc, bool sm = false);
const void *lean_kernel_heston(int fp64, int minb, bool stat, bool acc);
// The coarse paths of multilevel pairs (model: KX_MODEL_GBM or KX_MODEL_HESTON).
const void *lean_kernel_pair(int model, int fp64, bool stat, bool acc);

}  // namespace kx
