// paths_kernel.cuh — the fused path kernel (k_paths) and its launch layout.
//
// One kernel replaces Gbm::simulate / HestonSimulator::simulate
// (src/simulator.rs:215-253, 506-541) + price_on_paths / cashflows
// (src/pricer.rs:230-433): each thread draws its normals from Philox in
// registers, advances the path state (log-spot, variance) one grid step at a
// time and interprets the lowered contract table at every step, so the path is
// never stored. Only the discounted value of each path leaves the kernel.
//
// Scheduling: a persistent grid; each warp takes (contract, path-range) work
// items from an atomic counter and its 32 lanes take paths one by one from
// the item. A lane whose path finished early (every flow emitted or knocked
// out) starts a new path at once, so knocked-out barrier paths do not hold a
// lane idle. Per-path values go to fixed slots, so results do not depend on
// scheduling or on the launch variant.
//
// The kernel is instantiated in several translation units (paths_*.cu) at a
// few register budgets (MINB = minimum resident blocks per SM); the host
// autotuner picks the fastest variant.
#pragma once
#include <climits>

#include "device_common.cuh"

namespace kx {

constexpr int KX_MAX_NS = 7;
constexpr int KX_BLOCK = 256;

// ---------------------------------------------------------------------------
// device data layout
// ---------------------------------------------------------------------------
constexpr int KX_MAX_SPOT = KX_MAX_TRIG;

struct ContractDev {
    int32_t n_times;
    int32_t step_off;   // first StepRec of this contract
    int32_t disc_off;   // first discount factor (scenario s: + s * n_times)
    int32_t prog;       // index into the program array
    uint64_t n_paths;
    uint64_t pv_off;    // first output slot (scenario s: + s * pv_stride)
    uint64_t seed;
    uint32_t stream;    // Philox stream id
    int32_t smooth;     // 1: until(Spot cmp Const) is a logistic survival weight
    int32_t heston_scheme;
    int32_t uniform;    // every step k >= 1 has the same (c0, c1): uc0 / uc1
    double uc0, uc1;
    float uc0f, uc1f;
    // per-scenario values, in both precisions so the FP32 kernel never converts
    double s0[KX_MAX_NS], drift[KX_MAX_NS], sigma[KX_MAX_NS];
    float s0f[KX_MAX_NS], driftf[KX_MAX_NS], sigmaf[KX_MAX_NS];
    double v0, kappa, theta, sigma_v, rho, rho_perp, r, inv_w;
    float v0f, kappaf, thetaf, sigma_vf, rhof, rho_perpf, rf, inv_wf;
    uint32_t item_paths;  // paths per work item of this contract (arithmetic items) ...
    uint32_t item_big;    // ... for its first item_big items; the rest of item_small paths
    uint32_t item_small;  // (the launch's last contract ends in small items: a short tail)
    uint32_t path_base;   // index of its first path in the stream
    // M_MULTI: factors (s0 / drift / sigma above hold factor i at index i) and the
    // packed lower Cholesky factor of their correlation, row i at i (i + 1) / 2
    int32_t n_assets;
    double chol[KX_MAX_NS * (KX_MAX_NS + 1) / 2];
    float cholf[KX_MAX_NS * (KX_MAX_NS + 1) / 2];
};

struct WorkItem {
    int32_t contract;
    int32_t pad;
    uint64_t first;
    uint64_t count;
};

struct PathArgs {
    const KxProgram *progs;
    const void *steps;
    const double *disc;
    const ContractDev *cons;
    const void *thr;     // Real[contract][KX_MAX_NS][KX_MAX_SPOT] log-spot thresholds
    const WorkItem *items;
    uint32_t n_items;
    uint32_t slots;      // shared-memory slots per thread per scenario
    uint32_t surv_base;  // first survival slot (after 2 slots per accumulator)
    uint32_t pad;
    uint32_t *item_counter;
    uint32_t *err_word;
    unsigned long long *steps_done;
    double *pv;
    uint64_t pv_stride;
    const double *z64;   // shared draws (path-major) or null
    const float *z32;
    uint64_t z_dpp;
    const void *statics; // StaticDev per contract (static-schedule launches of k_lean)
    // Arithmetic work items (when `items` is null): the contracts in launch
    // order `item_order[0..n_order)`, contract item_order[q] owning items
    // item_start[q] .. item_start[q + 1] - 1 (item_big of item_paths paths,
    // then item_small paths each).
    const uint32_t *item_start;
    const int32_t *item_order;
    uint32_t n_order;
    // Philox round keys of the launch's seed when every contract of the
    // launch has the same seed (rk_ok), read as kernel parameters
    uint32_t rk_ok;
    uint32_t rk[20];
};

// Work item `it` of a launch: from the table, or computed from the
// contract's item size (no per-item table to build or upload).
__device__ __forceinline__ WorkItem fetch_item(const PathArgs &A, int it) {
    if (A.items) return A.items[it];
    int lo = 0, hi = (int)A.n_order - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.item_start[mid] <= (uint32_t)it) lo = mid;
        else hi = mid - 1;
    }
    const int c = A.item_order[lo];
    const ContractDev &C = A.cons[c];
    const uint32_t j = (uint32_t)it - A.item_start[lo];
    uint64_t local, cnt;
    if (j < C.item_big) {
        local = (uint64_t)j * C.item_paths;
        cnt = C.item_paths;
    } else {
        local = (uint64_t)C.item_big * C.item_paths + (uint64_t)(j - C.item_big) * C.item_small;
        cnt = C.item_small;
    }
    const uint64_t left = C.n_paths - local;
    return WorkItem{c, 0, (uint64_t)C.path_base + local, left < cnt ? left : cnt};
}

// Path models of k_paths. The _PAIR models are the coarse paths of a
// multilevel Monte-Carlo pair (simulator.rs:321-409, 592-690): every coarse
// step consumes the normals of two fine steps of the same Philox stream, so a
// coarse job on the seed and path indices of its fine job is coupled to it.
enum { M_GBM = 0, M_HESTON = 1, M_GBM_PAIR = 2, M_HESTON_PAIR = 3, M_MULTI = 4 };
// M_MULTI: n_assets correlated GBM factors (CorrelatedGbmN, multi_asset.rs:107-170):
// each step draws n_assets normals z, correlates them with the lower Cholesky
// factor (w = L z) and steps factor i with its own drift and volatility.

// Per-contract values a warp keeps in registers: only what the per-step hot
// path reads. Everything else is read from the (L1-resident) program table
// when something fires.
template <class Real, int NS>
struct Hot {
    const KxProgram *P;
    const StepRec<Real> *R;
    uint32_t fast_bit;   // the one Spot-cmp-Const slot checked from registers
    uint32_t gen_mask;   // price-dependent slots needing the interpreter
    uint32_t time_mask;
    uint32_t flags;      // HF_* below
    int n_times;
    int n_acc;
    uint32_t fast_kill;  // flows dropped when the fast slot is an until and knocks
    uint32_t all_leaves;
    int init_nte;
    Real fsign;          // y * fsign  >= / >  fthr[s]
    Real uc0, uc1;       // step coefficients of a uniform grid (HF_UNIFORM)
    Real fthr[NS];
    Real s0[NS];
};
enum : uint32_t {
    HF_SPOT_EACH = 1, HF_SMOOTH = 2, HF_STRICT = 4, HF_FULLTRUNC = 8, HF_UNIFORM = 16, HF_RARE_EACH = 32,
    HF_FAST_UNTIL = 64, HF_ERRCAP = 128, HF_ROOT_LEAVES = 256
};

template <class Real, int NS>
struct Lane {
    Real y[NS];  // log(S / s0) of each scenario
    Real v[NS];  // Heston variance
    uint32_t armed[NS], resolved[NS], dead[NS], emitted[NS], poisoned[NS];
    int nte[NS];  // next step at which a live time-only slot can change
    double pv[NS];
    uint32_t err;
};

template <class Real, int NS>
__device__ __forceinline__ void load_hot(Hot<Real, NS> &H, const PathArgs &A, int c) {
    const ContractDev *C = A.cons + c;
    H.P = A.progs + C->prog;
    H.R = reinterpret_cast<const StepRec<Real> *>(A.steps) + C->step_off;
    const Real *thr = reinterpret_cast<const Real *>(A.thr) + (size_t)c * KX_MAX_NS * KX_MAX_SPOT;
#pragma unroll
    for (int s = 0; s < NS; ++s) H.s0[s] = pick<Real>(C->s0[s], C->s0f[s]);
    H.n_times = C->n_times;
    const KxProgram &P = *H.P;
    H.n_acc = P.n_acc;
    H.time_mask = P.time_mask;
    H.flags = (P.spot_each_step ? HF_SPOT_EACH : 0u) | (C->smooth ? HF_SMOOTH : 0u) |
              (C->heston_scheme == KX_HESTON_FULL_TRUNCATION ? HF_FULLTRUNC : 0u) | (C->uniform ? HF_UNIFORM : 0u);
    H.uc0 = pick<Real>(C->uc0, C->uc0f);
    H.uc1 = pick<Real>(C->uc1, C->uc1f);
    H.fast_bit = 0;
    H.fast_kill = 0;
    H.all_leaves = P.all_leaves;
    H.init_nte = P.init_nte;
    if (P.err_capable) H.flags |= HF_ERRCAP;
    if (P.root_leaves) H.flags |= HF_ROOT_LEAVES;
    H.fsign = Real(1);
#pragma unroll
    for (int s = 0; s < NS; ++s) H.fthr[s] = Real(0);
    uint32_t pm = P.price_mask;
    if (C->smooth) pm &= ~P.until_mask;  // smoothed untils never knock
    uint32_t gen = pm;
    while (pm) {
        const int i = __ffs(pm) - 1;
        pm &= pm - 1;
        const KxTrig &T = P.trig[i];
        if (T.cond_kind == CK_SPOT_CMP) {
            H.fast_bit = 1u << i;
            gen &= ~H.fast_bit;
            if (T.cmp == CMP_GT || T.cmp == CMP_LT) H.flags |= HF_STRICT;
            if (T.kind == TK_UNTIL) {
                H.flags |= HF_FAST_UNTIL;
                H.fast_kill = T.leaves;
            }
            H.fsign = (T.cmp == CMP_LE || T.cmp == CMP_LT) ? Real(-1) : Real(1);
#pragma unroll
            for (int s = 0; s < NS; ++s) H.fthr[s] = H.fsign * thr[s * KX_MAX_SPOT + T.spot_slot];
            break;
        }
    }
    H.gen_mask = gen;
    if (gen || C->smooth) H.flags |= HF_RARE_EACH;
}

template <class Real>
__device__ __forceinline__ bool cmp_y(uint8_t cmp, Real y, Real thr) {
    switch (cmp) {
    case CMP_GE: return y >= thr;
    case CMP_GT: return y > thr;
    case CMP_LE: return y <= thr;
    default: return y < thr;
    }
}

// Survival weight of one step under a smoothed until(S cmp B): the breach
// indicator 1{y cmp b} is replaced by the logistic sigma(+-(y - b) / w)
// (smooth_weight: exactly 1 far inside the barrier).
template <class Real>
__device__ __forceinline__ Real smooth_survival(uint8_t cmp, Real y, Real thr, Real inv_w) {
    Real x = (y - thr) * inv_w;  // > 0 beyond the barrier for >=, >
    if (cmp == CMP_LE || cmp == CMP_LT) x = -x;
    return smooth_weight(x);
}

// Full condition evaluation of the slots in `mask` at step k: time bits from
// the table, Spot-cmp-Const from the thresholds, anything else through the
// expression interpreter.
template <class Real>
__device__ __forceinline__ uint32_t cond_bits_full(const KxProgram &P, const StepRec<Real> *R, const Real *thr,
                                                   bool smooth, Real y, Real S, uint32_t poisoned, uint32_t mask, int k,
                                                   AccView<Real> acc, uint32_t &err, const Real *Sx) {
    uint32_t bits = mask & P.time_mask;
    if (bits) bits &= R[k].tt;
    uint32_t pm = mask & ~P.time_mask;
    while (pm) {
        const int i = __ffs(pm) - 1;
        pm &= pm - 1;
        const KxTrig &T = P.trig[i];
        bool b;
        if (T.cond_kind == CK_SPOT_CMP) {
            if (smooth && T.kind == TK_UNTIL) continue;  // weighted instead of knocked
            b = cmp_y<Real>(T.cmp, y, thr[T.spot_slot]);
        } else {
            b = eval_code<Real>(P, T.code_off, T.code_len, acc, poisoned, k, S, err, Sx) != Real(0);
        }
        if (b) bits |= 1u << i;
    }
    return bits;
}

// Trigger state of one path and scenario, passed by value to the out-of-line
// event handler so that the kernel's registers never have their address taken.
struct Trig {
    uint32_t armed, resolved, dead, emitted, poisoned, err;
    int nte;
    int done;
    double pv;
};

// The rare part of a step, out of line: general conditions, smoothed
// weights, firing cascade, flows, next time event (pricer.rs:374-433).
// `bits` holds the live slots already known to fire at step k.
template <class Real>
__device__ __noinline__ Trig on_event(const KxProgram *Pp, const ContractDev *Cp, const StepRec<Real> *R,
                                      const Real *thr, const double *D, Real *acc_base, Real *surv_base, int stride,
                                      Real s0, Real y, int k, uint32_t bits, uint32_t gen_mask, int smooth, Trig st,
                                      const Real *Sx) {
    const KxProgram &P = *Pp;
    const AccView<Real> acc{acc_base, stride};
    const AccView<Real> surv{surv_base, stride};
    const Real inv_w = pick<Real>(Cp->inv_w, Cp->inv_wf);
    const Real S = spot_of<Real>(s0, y);
    const uint32_t live = st.armed & ~st.resolved;
    if (live & gen_mask)
        bits |= cond_bits_full<Real>(P, R, thr, smooth, y, S, st.poisoned, live & gen_mask, k, acc, st.err, Sx);
    if (smooth) {  // smoothed until weights of the slots armed before this step
        uint32_t sm = st.armed & P.until_mask & ~P.time_mask;
        while (sm) {
            const int i = __ffs(sm) - 1;
            sm &= sm - 1;
            const KxTrig &T = P.trig[i];
            if (T.cond_kind == CK_SPOT_CMP) surv[T.spot_slot] *= smooth_survival<Real>(T.cmp, y, thr[T.spot_slot], inv_w);
        }
    }
    if (!bits && k != 0) return st;
    uint32_t fired = 0;
    uint32_t newly = bits;
    while (newly) {
        st.resolved |= newly;
        uint32_t u = newly & P.until_mask;
        while (u) {
            const int i = __ffs(u) - 1;
            u &= u - 1;
            st.dead |= P.trig[i].leaves & ~st.emitted;
        }
        uint32_t w = newly & P.when_mask;
        fired |= w;
        uint32_t arm = 0;
        while (w) {
            const int i = __ffs(w) - 1;
            w &= w - 1;
            arm |= P.trig[i].fire_arm;
        }
        arm &= ~st.armed;
        st.armed |= arm;
        newly = arm ? cond_bits_full<Real>(P, R, thr, smooth, y, S, st.poisoned, arm, k, acc, st.err, Sx) : 0u;
        if (smooth && arm) {  // smoothed slots armed now weigh this step too
            uint32_t sm = arm & P.until_mask & ~P.time_mask;
            while (sm) {
                const int i = __ffs(sm) - 1;
                sm &= sm - 1;
                const KxTrig &T = P.trig[i];
                if (T.cond_kind == CK_SPOT_CMP) surv[T.spot_slot] *= smooth_survival<Real>(T.cmp, y, thr[T.spot_slot], inv_w);
            }
        }
    }
    // flows acquired at step k (pricer.rs:380-405)
    uint32_t acq = k == 0 ? P.root_leaves : 0u;
    while (fired) {
        const int i = __ffs(fired) - 1;
        fired &= fired - 1;
        acq |= P.trig[i].leaves;
    }
    acq &= ~st.emitted;
    while (acq) {
        const int j = __ffs(acq) - 1;
        acq &= acq - 1;
        const KxLeaf &F = P.leaf[j];
        const bool is_dead = (st.dead >> j) & 1u;
        if (is_dead && !F.err_capable) continue;
        double amt = F.kind == AK_CONST ? F.sign
                     : F.fast           ? (double)fast_amount<Real>(P, F, S)
                                        : (double)eval_code<Real>(P, F.code_off, F.code_len, acc, st.poisoned, k, S, st.err, Sx);
        if (is_dead) continue;
        if (smooth) {
            uint32_t us = P.until_mask & ~P.time_mask & st.armed;
            while (us) {
                const int i = __ffs(us) - 1;
                us &= us - 1;
                const KxTrig &T = P.trig[i];
                if (T.cond_kind == CK_SPOT_CMP && ((T.leaves >> j) & 1u)) amt *= (double)surv[T.spot_slot];
            }
        }
        st.pv = __dadd_rn(st.pv, __dmul_rn(amt, D[k]));
        st.emitted |= 1u << j;
    }
    // next step at which a live time-only slot can change
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
    st.done = !P.err_capable && (P.all_leaves & ~(st.emitted | st.dead)) == 0u;
    return st;
}

// Everything the contract does at grid step k for scenario s, after the
// model moved to step k. Returns true when no flow can change any more.
template <class Real, int NS>
__device__ __forceinline__ bool contract_step(const Hot<Real, NS> &H, const PathArgs &A, int cur, Lane<Real, NS> &L,
                                              int s, int k, Real *smem, const Real *Sx = nullptr) {
    const AccView<Real> acc{smem + (s * (int)A.slots) * KX_BLOCK + threadIdx.x, KX_BLOCK};
    if (H.n_acc) {  // accumulators (observable.rs:120-140), inner ones first (slot order)
        const KxProgram &P = *H.P;
        const Real S = spot_of<Real>(H.s0[s], L.y[s]);
        for (int a = 0; a < H.n_acc; ++a) {
            const KxAcc &Ac = P.acc[a];
            if (k < Ac.i_from || k > Ac.i_to) continue;
            Real x;
            if (Ac.inner == IK_SPOT) {
                x = Sx ? Sx[Ac.pad] : S;
            } else {
                uint32_t e = 0;
                x = eval_code<Real>(P, Ac.code_off, Ac.code_len, acc, L.poisoned[s], k, S, e, Sx);
                if (e) L.poisoned[s] |= 1u << a;
            }
            Real &v = acc[2 * a];
            if (Ac.kind == ACC_MAX) v = fmax(v, x);
            else if (Ac.kind == ACC_MIN) v = fmin(v, x);
            else if (sizeof(Real) == 8) v = v + x;
            else {  // compensated (Kahan) sum in FP32
                Real &c = acc[2 * a + 1];
                const Real yk = x - c;
                const Real t = v + yk;
                c = (t - v) - yk;
                v = t;
            }
        }
    }
    const uint32_t live = L.armed[s] & ~L.resolved[s];
    uint32_t bits = 0;
    if (live & H.fast_bit) {
        const Real yy = H.fsign * L.y[s];
        if ((H.flags & HF_STRICT) ? yy > H.fthr[s] : yy >= H.fthr[s]) bits = H.fast_bit;
    }
    if (k >= L.nte[s]) bits |= live & H.time_mask & H.R[k].tt;
    if (!(H.flags & HF_RARE_EACH)) {
        if (k == 0 && !bits && !(H.flags & HF_ROOT_LEAVES)) {  // nothing happens at t = 0
            L.nte[s] = H.init_nte;
            return false;
        }
        if (!bits && k != 0) return false;
        if (bits == H.fast_bit && (H.flags & HF_FAST_UNTIL) && k > 0) {  // barrier knock-out, inline
            L.resolved[s] |= bits;
            L.dead[s] |= H.fast_kill & ~L.emitted[s];
            return !(H.flags & HF_ERRCAP) && (H.all_leaves & ~(L.emitted[s] | L.dead[s])) == 0u;
        }
    }
    const ContractDev *C = A.cons + cur;
    Trig st{L.armed[s], L.resolved[s], L.dead[s], L.emitted[s], L.poisoned[s], L.err, L.nte[s], 0, L.pv[s]};
    st = on_event<Real>(H.P, C, H.R, reinterpret_cast<const Real *>(A.thr) + ((size_t)cur * KX_MAX_NS + s) * KX_MAX_SPOT,
                        A.disc + C->disc_off + (size_t)s * H.n_times, acc.base,
                        smem + (s * (int)A.slots + (int)A.surv_base) * KX_BLOCK + threadIdx.x, KX_BLOCK, H.s0[s],
                        L.y[s], k, bits, H.gen_mask, (H.flags & HF_SMOOTH) ? 1 : 0, st, Sx);
    L.armed[s] = st.armed;
    L.resolved[s] = st.resolved;
    L.dead[s] = st.dead;
    L.emitted[s] = st.emitted;
    L.poisoned[s] = st.poisoned;
    L.err = st.err;
    L.nte[s] = st.nte;
    L.pv[s] = st.pv;
    return st.done != 0;
}

template <class Real, int NS>
__device__ __forceinline__ void write_path(const PathArgs &A, int cur, int64_t path, const Lane<Real, NS> &L) {
    const uint64_t off = A.cons[cur].pv_off + (uint64_t)path;
#pragma unroll
    for (int s = 0; s < NS; ++s) A.pv[(uint64_t)s * A.pv_stride + off] = L.pv[s];
}

template <class Real, int MODEL, int NS, int MINB>
__global__ void __launch_bounds__(KX_BLOCK, MINB) k_paths(const PathArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *smem = reinterpret_cast<Real *>(smem_raw);
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    constexpr bool HESTON = MODEL == M_HESTON || MODEL == M_HESTON_PAIR;
    constexpr bool MULTI = MODEL == M_MULTI;  // one step per round, n_assets normals per step
    constexpr int DRAWS = MODEL == M_GBM ? 1 : MODEL == M_HESTON_PAIR || MULTI ? 4 : 2;  // normals per grid step
    constexpr int SPB = 4 / DRAWS;                                                       // grid steps per Philox block
    constexpr uint32_t ALL = (1u << NS) - 1u;

    // warp-uniform work state (path indices are per contract, < 2^32)
    int cur = -1, pend = -1;
    uint32_t nx = 0, end = 0;
    bool drained = false;
    Hot<Real, NS> H;
    Real hr = 0, hk = 0, hth = 0, hsv = 0, hrho = 0, hrp = 0, hv0 = 0;  // Heston parameters

    // lane state
    int64_t path = -1;
    int k = 0;
    uint32_t done = 0;
    Lane<Real, NS> L;
    L.err = 0;
    uint32_t my_steps = 0;
    int n_assets = 1;                      // warp-uniform (M_MULTI)
    Real ym[MULTI ? KX_MAX_NS : 1];        // M_MULTI: log(S_i / s0_i) of every factor
    Real sx[MULTI ? KX_MAX_NS : 1];        // M_MULTI: the factors' spots at the current step

    while (true) {
        // ---- hand paths to idle lanes (warp-uniform control) ----
        unsigned idle = __ballot_sync(FULL, path < 0);
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
                    load_hot<Real, NS>(H, A, cur);
                    if (MULTI) n_assets = A.cons[cur].n_assets;
                    if (HESTON) {
                        const ContractDev &C = A.cons[cur];
                        hr = pick<Real>(C.r, C.rf);
                        hk = pick<Real>(C.kappa, C.kappaf);
                        hth = pick<Real>(C.theta, C.thetaf);
                        hsv = pick<Real>(C.sigma_v, C.sigma_vf);
                        hrho = pick<Real>(C.rho, C.rhof);
                        hrp = pick<Real>(C.rho_perp, C.rho_perpf);
                        hv0 = pick<Real>(C.v0, C.v0f);
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
            if (path < 0 && rank < take) {
                path = (int64_t)(nx + (uint32_t)rank);
                // new path: state at t = 0 (S = s0), then the contract at step 0
                const KxProgram &P = *H.P;
                done = 0;
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    L.y[s] = Real(0);
                    L.v[s] = fmax(hv0, Real(0));
                    L.armed[s] = P.root_arm;
                    L.resolved[s] = L.dead[s] = L.emitted[s] = L.poisoned[s] = 0u;
                    L.nte[s] = 0;
                    L.pv[s] = 0.0;
                    AccView<Real> av{smem + (s * (int)A.slots) * KX_BLOCK + threadIdx.x, KX_BLOCK};
                    for (int a = 0; a < H.n_acc; ++a) {
                        av[2 * a] = P.acc[a].kind == ACC_MAX   ? Real(-INFINITY)
                                    : P.acc[a].kind == ACC_MIN ? Real(INFINITY)
                                                               : Real(0);
                        av[2 * a + 1] = Real(0);
                    }
                    if (H.flags & HF_SMOOTH)
                        for (int q = 0; q < P.n_spot_cmp; ++q) av[(int)A.surv_base + q] = Real(1);
                    if (MULTI) {
                        const ContractDev &C = A.cons[cur];
#pragma unroll
                        for (int i = 0; i < (MULTI ? KX_MAX_NS : 1); ++i) {
                            ym[i] = Real(0);
                            sx[i] = i < n_assets ? pick<Real>(C.s0[i], C.s0f[i]) : Real(0);
                        }
                    }
                    if (contract_step<Real, NS>(H, A, cur, L, s, 0, smem, MULTI ? sx : nullptr)) done |= 1u << s;
                }
                k = 1;
                if (H.n_times <= 1 || done == ALL) {
                    write_path<Real, NS>(A, cur, path, L);
                    path = -1;
                }
            }
            nx += (uint32_t)take;
            if (take == 0) break;
            idle = __ballot_sync(FULL, path < 0);
        }
        if (__ballot_sync(FULL, path >= 0) == 0u) {
            if (drained && pend < 0 && nx >= end) break;
            continue;
        }

        // ---- M_MULTI: advance busy lanes by one grid step of every factor ----
        if (MULTI && path >= 0) {
            const ContractDev &C = A.cons[cur];
            const int kk = k;
            Real c0, c1;
            if (H.flags & HF_UNIFORM) {
                c0 = H.uc0;
                c1 = H.uc1;
            } else {
                const StepRec<Real> rec = H.R[kk];
                c0 = rec.c0;
                c1 = rec.c1;
            }
            // the step's normals are draws (kk - 1) n .. (kk - 1) n + n - 1 of the path's stream;
            // the factor loops are unrolled over the largest count so the state stays in registers
            Real z[MULTI ? KX_MAX_NS : 1];
            const uint64_t d0 = (uint64_t)(kk - 1) * (uint64_t)n_assets;
            uint32_t blk = 0xffffffffu;
            Real zz[4] = {Real(0), Real(0), Real(0), Real(0)};
#pragma unroll
            for (int i = 0; i < (MULTI ? KX_MAX_NS : 1); ++i) {
                z[i] = Real(0);
                if (i < n_assets) {
                    const uint64_t d = d0 + (uint64_t)i;
                    if (A.z64 == nullptr && A.z32 == nullptr) {
                        if ((uint32_t)(d >> 2) != blk) {
                            blk = (uint32_t)(d >> 2);
                            const uint4 w = philox4x32_10(
                                make_uint4(blk, (uint32_t)path, (uint32_t)((uint64_t)path >> 32), C.stream),
                                (uint32_t)C.seed, (uint32_t)(C.seed >> 32));
                            box_muller(w.x, w.y, zz[0], zz[1]);
                            box_muller(w.z, w.w, zz[2], zz[3]);
                        }
                        const uint32_t q = (uint32_t)(d & 3);
                        z[i] = q == 0 ? zz[0] : q == 1 ? zz[1] : q == 2 ? zz[2] : zz[3];
                    } else {
                        const uint64_t base = (uint64_t)path * A.z_dpp;
                        z[i] = d < A.z_dpp ? (A.z64 ? (Real)A.z64[base + d] : (Real)A.z32[base + d]) : Real(0);
                    }
                }
            }
            // w = L z (multi_asset.rs:146-156), then each factor's exact log step
#pragma unroll
            for (int i = 0; i < (MULTI ? KX_MAX_NS : 1); ++i) {
                if (i < n_assets) {
                    Real wi = Real(0);
                    const int row = i * (i + 1) / 2;
#pragma unroll
                    for (int j = 0; j <= i; ++j) wi = wi + pick<Real>(C.chol[row + j], C.cholf[row + j]) * z[j];
                    ym[i] = gbm_step(ym[i], pick<Real>(C.drift[i], C.driftf[i]) * c0,
                                     pick<Real>(C.sigma[i], C.sigmaf[i]) * c1, wi);
                    sx[i] = spot_of<Real>(pick<Real>(C.s0[i], C.s0f[i]), ym[i]);
                }
            }
            L.y[0] = ym[0];
            if (contract_step<Real, NS>(H, A, cur, L, 0, kk, smem, sx)) done = ALL;
            ++my_steps;
            k += 1;
            if (k >= H.n_times || done == ALL) {
                write_path<Real, NS>(A, cur, path, L);
                path = -1;
            }
        }
        // ---- advance busy lanes by one Philox block of grid steps ----
        if (!MULTI && path >= 0) {
            const int nt = H.n_times;
            Real zz[4];
            if (A.z64 == nullptr && A.z32 == nullptr) {
                const ContractDev &C = A.cons[cur];
                const uint32_t blk = (uint32_t)((k - 1) / SPB);
                const uint4 w = philox4x32_10(make_uint4(blk, (uint32_t)path, (uint32_t)((uint64_t)path >> 32), C.stream),
                                              (uint32_t)C.seed, (uint32_t)(C.seed >> 32));
                box_muller(w.x, w.y, zz[0], zz[1]);
                box_muller(w.z, w.w, zz[2], zz[3]);
            } else {
                const uint64_t d0 = (uint64_t)(k - 1) * DRAWS;
                const uint64_t base = (uint64_t)path * A.z_dpp + d0;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    zz[j] = d0 + j < A.z_dpp ? (A.z64 ? (Real)A.z64[base + j] : (Real)A.z32[base + j]) : Real(0);
            }
#pragma unroll
            for (int j = 0; j < SPB; ++j) {
                const int kk = k + j;
                if (kk < nt && done != ALL) {
                    Real c0, c1;
                    if (H.flags & HF_UNIFORM) {
                        c0 = H.uc0;
                        c1 = H.uc1;
                    } else {
                        const StepRec<Real> rec = H.R[kk];
                        c0 = rec.c0;
                        c1 = rec.c1;
                    }
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        if ((done >> s) & 1u) continue;
                        if (!HESTON) {
                            // log-space exact GBM step (simulator.rs:238-245); a coarse step of a
                            // multilevel pair adds its two fine normals (simulator.rs:373-377)
                            const Real z = MODEL == M_GBM_PAIR ? zz[2 * j] + zz[2 * j + 1] : zz[j];
                            if (NS == 1) {
                                L.y[s] = gbm_step(L.y[s], c0, c1, z);
                            } else {
                                const ContractDev &C = A.cons[cur];
                                const Real sc1 = pick<Real>(C.sigma[s], C.sigmaf[s]) * c1;
                                L.y[s] = gbm_step(L.y[s], pick<Real>(C.drift[s], C.driftf[s]) * c0, sc1, z);
                            }
                        } else {
                            Real z1 = zz[2 * j], z2 = zz[2 * j + 1];
                            if (MODEL == M_HESTON_PAIR) {  // the two fine (z1, z2) pairs, summed over sqrt 2 (:656-661)
                                const Real inv_sqrt2 = Real(0.70710678118654752440);
                                z1 = (zz[0] + zz[2]) * inv_sqrt2;
                                z2 = (zz[1] + zz[3]) * inv_sqrt2;
                            }
                            heston_step<Real>(hr, hk, hth, hsv, hrho, hrp,
                                              (H.flags & HF_FULLTRUNC) ? KX_HESTON_FULL_TRUNCATION
                                                                       : KX_HESTON_REFERENCE_FLOOR,
                                              c0, c1, z1, z2, L.y[s], L.v[s]);
                        }
                        if (contract_step<Real, NS>(H, A, cur, L, s, kk, smem)) done |= 1u << s;
                    }
                    ++my_steps;
                }
            }
            k += SPB;
            if (k >= nt || done == ALL) {
                write_path<Real, NS>(A, cur, path, L);
                path = -1;
            }
        }
    }
    // counters: one atomic per warp
    unsigned long long tot = (unsigned long long)my_steps;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
    uint32_t err = L.err;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) err |= __shfl_xor_sync(FULL, err, o);
    if (lane == 0) {
        if (tot) atomicAdd(A.steps_done, tot);
        if (err) atomicOr(A.err_word, err);
    }
}

// Kernel variants, one function per translation unit.
// paths_kernel_pair: the coarse kernels of multilevel pairs (model 0 GBM, 1 Heston).
const void *paths_kernel_pair(int model, int fp64);
// paths_kernel_multi: correlated multi-factor GBM (M_MULTI) at a register budget.
const void *paths_kernel_multi(int fp64, int minb);
// paths_kernel_gbm / _heston: one scenario at a register budget (MINB).
const void *paths_kernel_gbm(int fp64, int minb);
const void *paths_kernel_heston(int fp64, int minb);

}  // namespace kx
