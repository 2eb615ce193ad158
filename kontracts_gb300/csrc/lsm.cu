// lsm.cu — Longstaff-Schwartz American pricing on the GPU
// (price_american_lsm / backward_induction, src/lsm.rs:80-229).
//
//  1. k_lsm_forward simulates every path on the grid [0, dates...] (the same
//     Philox counters as the European kernels, so the same paths) and stores
//     S at each exercise date in HBM, date-major: S[d * n_paths + i], so that
//     consecutive threads write and read consecutive addresses.
//  2. k_lsm_backward, one cooperative launch (every block resident), walks
//     the exercise dates backwards for every case of the call. Iteration it
//     applies the exercise decision of date d = n_ex - 1 - it to every path's
//     realised value (lsm.rs:196-222) and, in the same pass, accumulates the
//     normal equations A^T A, A^T y of date d - 1 over the in-the-money paths
//     (lsm.rs:259-288). Paths are cut into fixed tiles; each tile's sums go to
//     a fixed slot, the last tile to finish adds them in tile order
//     (deterministic, independent of the grid), solves the m x m system
//     (numerics.rs:190-236) and publishes the coefficients; the tiles of the
//     next date of that case wait for them (bounded waits). The last
//     iteration discounts the values to t = 0; the per-path values then go
//     through the same deterministic statistics as every price.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "device_common.cuh"
#include "ffloat.cuh"
#include "engine.hpp"

namespace kx {

constexpr int LSM_BLOCK = 256;
// Block reduction scratch (doubles): red[q * 8 + w] the 8 warps' sums of up to
// 32 quantities q, the block's sums at red[LSM_RED_OUT + q].
constexpr int LSM_RED_OUT = (LSM_BLOCK / 32) * 32;
constexpr int LSM_MAXM = 6;
constexpr int LSM_COEF = 12;  // coef[d * LSM_COEF + j], j < m; [7] = have-fit flag; doubles 8..11 hold
                              // the coefficients and the flag as floats (float index j, 7)

// The payoff as up to 4 closed-form terms (kinds FA_*, FA_NONE = the constant
// sign), in both precisions, converted once on the host.
struct LsmPayTab {
    int ok, n;
    uint8_t kind[4];
    double kd[4], sd[4];
    float kf[4], sf[4];
};

struct LsmArgs {
    const KxProgram *P;  // bound payoff program (root flows only)
    const void *steps;   // StepRec<Real>[n_times]
    const double *disc;  // disc[d] = exp(-rate (t_{d+1} - t_d)), d < n_ex - 1; disc[n_ex - 1] = exp(-rate t_0)
    int n_times;         // 1 + n_ex
    int n_ex;
    uint64_t n_paths;
    uint64_t seed;
    int model;
    int scheme;
    double s0, v0, kappa, theta, sigma_v, rho, rho_perp, r;
    double x_scale;    // regressor x = S / x_scale (the model's spot): Laguerre basis, FP32 fits
    // the same parameters rounded to FP32 on the host (GB300's FP64 pipe runs
    // at ~1/64 of FP32: no thread converts a double), inv_scale_f = 1 / x_scale
    float s0_f, v0_f, kappa_f, theta_f, sigma_v_f, rho_f, rho_perp_f, r_f, inv_scale_f;
    const float *disc_f;  // (float) disc[d]
    LsmPayTab pay;
    const double *z64;
    const float *z32;
    uint64_t z_dpp;
    void *S;           // Real[n_ex][ld]
    uint64_t ld;       // row stride of S: n_paths rounded up to 64 (every row 256-byte aligned)
    void *value;       // Real[n_paths]: realised value at the current date
    double *pv;        // final per-path values
    double *partial;   // [n_tiles][LSM_NSUM]: a tile's normal equations
    double *coef;      // [n_ex][LSM_COEF]
    unsigned *sync;    // [0] iterations solved and published, [1] tiles of the current iteration done
    unsigned n_tiles;
};

// Value of the exercised contract at exercise step k (lsm.rs:238-251): the
// lowered payoff has only flows acquired at once, so each flow's discount to
// the exercise date is exp(0) = 1 and the value is the sum of the amounts.
template <class Real>
__device__ __forceinline__ Real lsm_payoff(const KxProgram &P, Real S, int k) {
    Real v = Real(0);
    AccView<Real> none{nullptr, 0};
    for (int j = 0; j < P.n_leaf; ++j) {
        const KxLeaf &F = P.leaf[j];
        uint32_t e = 0;
        v += F.kind == AK_CONST ? (Real)F.sign
             : F.fast           ? fast_amount<Real>(P, F, S)
                                : eval_code<Real>(P, F.code_off, F.code_len, none, 0u, k, S, e);
    }
    return v;
}

// The payoff as up to 4 closed-form terms in the path precision, converted
// once per thread (no double is converted per path on GB300's slow FP64
// pipe); `ok` is false when some term needs the interpreter.
template <class Real>
struct LsmPay {
    bool ok;
    int n;
    uint8_t kind[4];  // FA_NONE: the constant sign[q]
    Real k[4], sign[4];
};

// Host side: the closed-form terms of a bound payoff program.
inline LsmPayTab lsm_pay_tab(const KxProgram &P) {
    LsmPayTab t{};
    t.ok = P.n_leaf <= 4;
    t.n = 0;
    for (int j = 0; j < P.n_leaf && t.ok; ++j) {
        const KxLeaf &F = P.leaf[j];
        if (F.kind != AK_CONST && !F.fast) t.ok = false;
        t.kind[t.n] = F.kind == AK_CONST ? (uint8_t)FA_NONE : F.fast;
        t.kd[t.n] = F.kind == AK_CONST ? 0.0 : P.cpool[F.fast_k];
        t.sd[t.n] = (double)F.sign;
        t.kf[t.n] = (float)t.kd[t.n];
        t.sf[t.n] = (float)t.sd[t.n];
        ++t.n;
    }
    return t;
}

template <class Real>
__device__ __forceinline__ Real pick(double d, float f) {
    if constexpr (sizeof(Real) == 4) return f;
    else return d;
}

template <class Real>
__device__ __forceinline__ LsmPay<Real> lsm_pay_terms(const LsmPayTab &T) {
    LsmPay<Real> t;
    t.ok = T.ok;
    t.n = T.n;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        t.kind[q] = T.kind[q];
        t.k[q] = pick<Real>(T.kd[q], T.kf[q]);
        t.sign[q] = pick<Real>(T.sd[q], T.sf[q]);
    }
    return t;
}

// lsm_payoff by the closed-form terms (the same operations as fast_amount).
template <class Real>
__device__ __forceinline__ Real lsm_payoff_terms(const LsmPay<Real> &t, Real S) {
    Real v = Real(0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (q >= t.n) break;
        Real r;
        switch (t.kind[q]) {
        case FA_NONE: v += t.sign[q]; continue;
        case FA_CALL: r = fmax(S - t.k[q], Real(0)); break;
        case FA_PUT: r = fmax(t.k[q] - S, Real(0)); break;
        case FA_SPOT: r = S; break;
        default: r = t.k[q]; break;
        }
        v += t.sign[q] < Real(0) ? -r : r;
    }
    return v;
}

template <class Real>
__device__ __forceinline__ Real lsm_pay(const LsmPay<Real> &t, const KxProgram &P, Real S, int k) {
    return t.ok ? lsm_payoff_terms<Real>(t, S) : lsm_payoff<Real>(P, S, k);
}

// The same with the choice made by the caller (GEN: the interpreter), so
// that a kernel specialised for closed-form payoffs contains no call.
template <class Real, bool GEN>
__device__ __forceinline__ Real lsm_pay_g(const LsmPay<Real> &t, const KxProgram &P, Real S, int k) {
    if constexpr (GEN) return lsm_payoff<Real>(P, S, k);
    else return lsm_payoff_terms<Real>(t, S);
}

template <class Real, int MODEL>
__global__ void __launch_bounds__(LSM_BLOCK) k_lsm_forward(const LsmArgs A) {
    constexpr int DRAWS = MODEL == KX_MODEL_GBM ? 1 : 2;
    const StepRec<Real> *R = reinterpret_cast<const StepRec<Real> *>(A.steps);
    Real *S = reinterpret_cast<Real *>(A.S);
    const Real s0 = pick<Real>(A.s0, A.s0_f), r = pick<Real>(A.r, A.r_f), kap = pick<Real>(A.kappa, A.kappa_f),
               th = pick<Real>(A.theta, A.theta_f), sv = pick<Real>(A.sigma_v, A.sigma_v_f),
               rho = pick<Real>(A.rho, A.rho_f), rp = pick<Real>(A.rho_perp, A.rho_perp_f);
    const Real v_init = pick<Real>(fmax(A.v0, 0.0), A.v0_f);  // v0_f = max(v0, 0) in FP32
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < A.n_paths;
         i += (uint64_t)gridDim.x * blockDim.x) {
        Real y = Real(0), v = v_init;
        Real z[4];
        for (int k = 1; k < A.n_times; ++k) {
            const uint64_t d = (uint64_t)(k - 1) * DRAWS;
            if ((d & 3u) == 0) {
                if (A.z64 == nullptr && A.z32 == nullptr) {
                    const uint4 w = philox4x32_10(make_uint4((uint32_t)(d >> 2), (uint32_t)i, (uint32_t)(i >> 32), 0u),
                                                  (uint32_t)A.seed, (uint32_t)(A.seed >> 32));
                    box_muller(w.x, w.y, z[0], z[1]);
                    box_muller(w.z, w.w, z[2], z[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        z[j] = d + j < A.z_dpp ? (A.z64 ? (Real)A.z64[i * A.z_dpp + d + j] : (Real)A.z32[i * A.z_dpp + d + j])
                                               : Real(0);
                }
            }
            const StepRec<Real> rec = R[k];
            const int q = (int)(d & 3u);
            if (MODEL == KX_MODEL_GBM) {
                y = gbm_step(y, rec.c0, rec.c1, z[q]);
            } else {
                heston_step<Real>(r, kap, th, sv, rho, rp, A.scheme, rec.c0, rec.c1, z[q], z[q + 1], y, v);
            }
            S[(uint64_t)(k - 1) * A.ld + i] = s0 * fast_exp<Real>(y);
        }
    }
}

// k_lsm_forward for FP32 paths: thread t simulates the four consecutive paths
// 4t .. 4t + 3 side by side (four independent Philox chains per thread) and
// stores their spots at each date with one 16-byte store: rows of S are
// padded to 64 elements (256 bytes), so S + d * ld + 4t is 16-byte aligned,
// and a row's padding past n_paths absorbs the last group's extra lanes.
// Every path's spots are those of k_lsm_forward<float> bit for bit (the same
// operations on the same draws).
template <int MODEL>
__global__ void __launch_bounds__(LSM_BLOCK) k_lsm_forward4(const LsmArgs A) {
    constexpr int DRAWS = MODEL == KX_MODEL_GBM ? 1 : 2;
    const StepRec<float> *R = reinterpret_cast<const StepRec<float> *>(A.steps);
    float *S = reinterpret_cast<float *>(A.S);
    const float s0 = A.s0_f, r = A.r_f, kap = A.kappa_f, th = A.theta_f, sv = A.sigma_v_f, rho = A.rho_f,
                rp = A.rho_perp_f;
    const float v_init = A.v0_f;  // max(v0, 0) in FP32
    const uint64_t n_groups = (A.n_paths + 3) / 4;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < n_groups;
         g += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i0 = 4 * g;
        float y[4] = {0.f, 0.f, 0.f, 0.f}, v[4] = {v_init, v_init, v_init, v_init};
        constexpr int SPB = 4 / DRAWS;  // steps per Philox block
        const int n_steps = A.n_times - 1;
        for (int kb = 0; kb < n_steps; kb += SPB) {  // steps kb + 1 .. kb + SPB
            const uint64_t d = (uint64_t)kb * DRAWS;  // the block's first draw (a multiple of 4)
            float z[4][4];
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const uint64_t i = i0 + p;
                if (A.z64 == nullptr && A.z32 == nullptr) {
                    const uint4 w = philox4x32_10(make_uint4((uint32_t)(d >> 2), (uint32_t)i, (uint32_t)(i >> 32), 0u),
                                                  (uint32_t)A.seed, (uint32_t)(A.seed >> 32));
                    box_muller(w.x, w.y, z[p][0], z[p][1]);
                    box_muller(w.z, w.w, z[p][2], z[p][3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        z[p][j] = i < A.n_paths && d + j < A.z_dpp
                                      ? (A.z64 ? (float)A.z64[i * A.z_dpp + d + j] : A.z32[i * A.z_dpp + d + j])
                                      : 0.f;
                }
            }
#pragma unroll
            for (int j = 0; j < SPB; ++j) {
                const int k = kb + 1 + j;
                if (k > n_steps) break;
                const StepRec<float> rec = R[k];
                float4 out;
                float *o = &out.x;
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    if (MODEL == KX_MODEL_GBM) {
                        y[p] = gbm_step(y[p], rec.c0, rec.c1, z[p][j]);
                    } else {
                        heston_step<float>(r, kap, th, sv, rho, rp, A.scheme, rec.c0, rec.c1, z[p][2 * j],
                                           z[p][2 * j + 1], y[p], v[p]);
                    }
                    o[p] = s0 * fast_exp<float>(y[p]);
                }
                *reinterpret_cast<float4 *>(S + (uint64_t)(k - 1) * A.ld + i0) = out;
            }
        }
    }
}

// Block-wide sum of `n` <= 32 doubles per thread into red[LSM_RED_OUT + q]
// (fixed order).
__device__ void block_sums(double *vals, int n, double *red) {
    static_assert(LSM_BLOCK == 256, "8 warps");
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int q = 0; q < n; ++q) {
        double v = vals[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0) red[q * 8 + w] = v;
    }
    __syncthreads();
    if (threadIdx.x < n) {
        double t = 0.0;
        for (int j = 0; j < nw; ++j) t += red[threadIdx.x * 8 + j];
        red[LSM_RED_OUT + threadIdx.x] = t;
    }
    __syncthreads();
}

// FP32 partial sums of a block in float-float: each warp adds its 32 lanes in
// FP32 (fixed xor tree), the 8 warps' totals are added in float-float in a
// fixed tree; sum q lands in out[q].
__device__ void block_sums_ff(const float *vals, int n, double *red, ff *out) {
    static_assert(LSM_BLOCK == 256, "8 warps: a 3-level tree");
    float *rf = reinterpret_cast<float *>(red);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int q = 0; q < n; ++q) {
        float v = vals[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0) rf[q * 8 + w] = v;
    }
    __syncthreads();
    if (threadIdx.x < n) {
        const float *r = rf + threadIdx.x * 8;
        const ff a = ff_add(two_sum(r[0], r[1]), two_sum(r[2], r[3]));
        const ff b = ff_add(two_sum(r[4], r[5]), two_sum(r[6], r[7]));
        out[threadIdx.x] = ff_add(a, b);
    }
    __syncthreads();
}

// Regression basis at spot s: monomials 1, s, ..., s^(M-1) (lsm.rs:273-278),
// or weighted Laguerre polynomials e^(-x/2) L_j(x), x = s / x_scale, with
// L_0 = 1, L_1 = 1 - x, (j + 1) L_(j+1) = (2j + 1 - x) L_j - j L_(j-1).
// Every product and sum is rounded separately (no FMA), as on the host.
template <int M, int B>
__device__ __forceinline__ void lsm_basis(double s, double x_scale, double (&phi)[M]) {
    if (B == KX_LSM_MONOMIAL) {
        phi[0] = 1.0;
#pragma unroll
        for (int j = 1; j < M; ++j) phi[j] = __dmul_rn(phi[j - 1], s);
    } else {
        const double x = __ddiv_rn(s, x_scale);
        const double w = exp(__dmul_rn(-0.5, x));
        double lm = 1.0, l = __dsub_rn(1.0, x);
        phi[0] = w;
        if (M > 1) phi[1] = __dmul_rn(w, l);
#pragma unroll
        for (int j = 1; j + 1 < M; ++j) {
            const double ln = __ddiv_rn(__dsub_rn(__dmul_rn(__dsub_rn((double)(2 * j + 1), x), l), __dmul_rn((double)j, lm)),
                                        (double)(j + 1));
            lm = l;
            l = ln;
            phi[j + 1] = __dmul_rn(w, l);
        }
    }
}

// FP32 paths: the basis of x = s / x_scale in FP32 (monomials x^j or the
// weighted Laguerre functions); the regression is invariant to the scale, so
// the fitted continuation is that of the reference's basis, while FP32 keeps
// the per-path work off the slow FP64 pipe. FP64 is used only across threads
// (block sums, cross-block sums) and for the solve.
template <int M, int B>
__device__ __forceinline__ void lsm_basis_f32(float x, float (&phi)[M]) {
    if (B == KX_LSM_MONOMIAL) {
        phi[0] = 1.0f;
#pragma unroll
        for (int j = 1; j < M; ++j) phi[j] = phi[j - 1] * x;
    } else {
        const float w = __expf(-0.5f * x);
        float lm = 1.0f, l = 1.0f - x;
        phi[0] = w;
        if (M > 1) phi[1] = w * l;
#pragma unroll
        for (int j = 1; j + 1 < M; ++j) {
            const float ln = (((float)(2 * j + 1) - x) * l - (float)j * lm) * (1.0f / (float)(j + 1));
            lm = l;
            l = ln;
            phi[j + 1] = w * l;
        }
    }
}

// Continuation value sum_j c_j phi_j(s): Horner from the top coefficient for
// monomials (poly_eval, lsm.rs:293-295), the plain sum for Laguerre.
template <int M, int B>
__device__ __forceinline__ double lsm_continuation(const double (&c)[M], double s, double x_scale) {
    double cont = 0.0;
    if (B == KX_LSM_MONOMIAL) {
#pragma unroll
        for (int j = M - 1; j >= 0; --j) cont = __dadd_rn(__dmul_rn(cont, s), c[j]);
    } else {
        double phi[M];
        lsm_basis<M, B>(s, x_scale, phi);
#pragma unroll
        for (int j = 0; j < M; ++j) cont = __dadd_rn(cont, __dmul_rn(c[j], phi[j]));
    }
    return cont;
}

// numerics.rs:190-236 (Gauss elimination with partial pivoting, a pivot below
// 1e-12 gives zero coefficients) for M <= LSM_MAXM on one warp: lane r < M
// holds row r of [A | b] in registers. Every element goes through the
// serial algorithm's operations in its order (each product and difference
// rounded separately, as on the host), and every lane runs the serial pivot
// search on the same values; the rows below a pivot are eliminated in
// parallel. Called by all 32 lanes of a warp.
template <int M>
__device__ void solve_gauss_warp(const double *red, int NA, double (&x)[LSM_MAXM]) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    double a[M], b = 0.0;
#pragma unroll
    for (int c = 0; c < M; ++c) a[c] = 0.0;
    if (lane < M) {  // row `lane` of the symmetric matrix from its upper triangle
        int q = 0;
#pragma unroll
        for (int r = 0; r < M; ++r)
#pragma unroll
            for (int c = r; c < M; ++c) {
                if (r == lane) a[c] = red[q];
                if (c == lane) a[r] = red[q];
                ++q;
            }
        b = red[NA + lane];
    }
    bool singular = false;
#pragma unroll
    for (int col = 0; col < M; ++col) {
        // pivot: the first row from col on with the largest |a[row][col]|
        int piv = col;
        double best = fabs(__shfl_sync(FULL, a[col], col));
#pragma unroll
        for (int row = col + 1; row < M; ++row) {
            const double v = fabs(__shfl_sync(FULL, a[col], row));
            if (v > best) { best = v; piv = row; }
        }
        if (best < 1e-12) { singular = true; break; }
        // swap rows col and piv
        double pr[M];
#pragma unroll
        for (int c = 0; c < M; ++c) {
            const double from_piv = __shfl_sync(FULL, a[c], piv), from_col = __shfl_sync(FULL, a[c], col);
            if (lane == col) a[c] = from_piv;
            else if (lane == piv) a[c] = from_col;
            pr[c] = from_piv;  // the pivot row after the swap
        }
        {
            const double bp = __shfl_sync(FULL, b, piv), bc = __shfl_sync(FULL, b, col);
            if (lane == col) b = bp;
            else if (lane == piv) b = bc;
        }
        const double bpiv = __shfl_sync(FULL, b, col);
        if (lane > col && lane < M) {
            const double factor = __ddiv_rn(a[col], pr[col]);
#pragma unroll
            for (int c = col; c < M; ++c) a[c] = __dsub_rn(a[c], __dmul_rn(factor, pr[c]));
            b = __dsub_rn(b, __dmul_rn(factor, bpiv));
        }
    }
    if (singular) {
#pragma unroll
        for (int j = 0; j < M; ++j) x[j] = 0.0;
        return;
    }
    // back substitution from the last row up (the same order of terms)
#pragma unroll
    for (int row = M - 1; row >= 0; --row) {
        double xr = 0.0;
        if (lane == row) {
            double sum = b;
#pragma unroll
            for (int c = row + 1; c < M; ++c) sum = __dsub_rn(sum, __dmul_rn(a[c], x[c]));
            xr = __ddiv_rn(sum, a[row]);
        }
        x[row] = __shfl_sync(FULL, xr, row);
    }
}

// solve_gauss_warp in float-float (the FP32 path mode): the same algorithm
// and order of operations, every element a float-float (48-bit significand)
// instead of a double, so that the chain of dependent divisions and products
// runs on the FP32 pipe (GB300's FP64 pipe issues at ~1/64 of the FP32 rate).
// The normal equations of this mode are summed in FP32 per thread and in
// float-float across threads, so the solve keeps their accuracy.
template <int M>
__device__ void solve_gauss_warp_ff(const ff *red, int NA, ff (&x)[LSM_MAXM]) {
    const int lane = threadIdx.x & 31;
    ff a[M], b = ff{0.0f, 0.0f};
#pragma unroll
    for (int c = 0; c < M; ++c) a[c] = ff{0.0f, 0.0f};
    if (lane < M) {  // row `lane` of the symmetric matrix from its upper triangle
        int q = 0;
#pragma unroll
        for (int r = 0; r < M; ++r)
#pragma unroll
            for (int c = r; c < M; ++c) {
                if (r == lane) a[c] = red[q];
                if (c == lane) a[r] = red[q];
                ++q;
            }
        b = red[NA + lane];
    }
    bool singular = false;
#pragma unroll
    for (int col = 0; col < M; ++col) {
        int piv = col;
        ff best = ff_abs(ff_shfl(a[col], col));
#pragma unroll
        for (int row = col + 1; row < M; ++row) {
            const ff v = ff_abs(ff_shfl(a[col], row));
            if (ff_gt(v, best)) { best = v; piv = row; }
        }
        if (best.hi < 1e-12f) { singular = true; break; }
        ff pr[M];
#pragma unroll
        for (int c = 0; c < M; ++c) {
            const ff from_piv = ff_shfl(a[c], piv), from_col = ff_shfl(a[c], col);
            if (lane == col) a[c] = from_piv;
            else if (lane == piv) a[c] = from_col;
            pr[c] = from_piv;
        }
        {
            const ff bp = ff_shfl(b, piv), bc = ff_shfl(b, col);
            if (lane == col) b = bp;
            else if (lane == piv) b = bc;
        }
        const ff bpiv = ff_shfl(b, col);
        if (lane > col && lane < M) {
            const ff factor = ff_div(a[col], pr[col]);
#pragma unroll
            for (int c = col; c < M; ++c) a[c] = ff_sub(a[c], ff_mul(factor, pr[c]));
            b = ff_sub(b, ff_mul(factor, bpiv));
        }
    }
    if (singular) {
#pragma unroll
        for (int j = 0; j < LSM_MAXM; ++j) x[j] = ff{0.0f, 0.0f};
        return;
    }
#pragma unroll
    for (int row = M - 1; row >= 0; --row) {
        ff xr = ff{0.0f, 0.0f};
        if (lane == row) {
            ff sum = b;
#pragma unroll
            for (int c = row + 1; c < M; ++c) sum = ff_sub(sum, ff_mul(a[c], x[c]));
            xr = ff_div(sum, a[row]);
        }
        x[row] = ff_shfl(xr, row);
    }
}

// Tiles: the paths of a case are cut into tiles of LSM_TILE consecutive
// paths (FP32: in sub-chunks of 4 * LSM_BLOCK paths, thread j takes the 4
// consecutive paths 4j .. 4j + 3 of each; FP64: thread j takes paths j,
// j + LSM_BLOCK, ...); a tile's
// normal equations are reduced in a fixed order (FP32 per thread and across a
// warp's lanes, FP64 across warps) and the tiles are added in tile order. The
// order depends only on the path count, so one case alone and in a batch, on
// any grid, gives the same bits.
constexpr int LSM_PPT = 32;
constexpr unsigned LSM_TILE = LSM_BLOCK * LSM_PPT;
constexpr int LSM_NSUM = 32;                    // stride of a partial (>= m(m+1)/2 + m + 1 for m <= 6)
constexpr unsigned LSM_SPIN_LIMIT = 1u << 22;   // polls of a wait (32 ns apart at least) before giving up;
                                                // KX_LSM_SPIN_LIMIT in the environment overrides it (tests)
constexpr int LSM_MAX_CASES = 1024;             // cases of one backward launch
constexpr int LSM_MAX_COORD = 16;               // coordinator blocks of one backward launch

inline unsigned lsm_tiles(uint64_t n_paths) { return (unsigned)((n_paths + LSM_TILE - 1) / LSM_TILE); }

// Sum q < NS of the rows src[b * LSM_NSUM + q], b < n, in a fixed order: T
// threads per sum (16 when 16 sums fit the block, else 8), thread t adds rows
// t, t + T, ... into 4 interleaved FP64 chains (GB300's FP64 pipe is slow;
// independent chains keep it busy), then the 4 chains and the T threads in a
// fixed tree. Called by the whole block; the sums land in dst[q] (shared).
template <int NS>
__device__ __forceinline__ void lsm_sum_rows(const double *src, unsigned n, double *dst) {
    constexpr int T = NS * 16 <= LSM_BLOCK ? 16 : 8;
    static_assert(NS * T <= LSM_BLOCK, "threads per sum");
    const int q = threadIdx.x / T, t = threadIdx.x % T;
    double s4[4] = {0.0, 0.0, 0.0, 0.0};
    if (q < NS) {
        unsigned b = t;
        for (; b + 3 * T < n; b += 4 * T) {
#pragma unroll
            for (int u = 0; u < 4; ++u) s4[u] += __ldcg(src + (size_t)(b + T * u) * LSM_NSUM + q);
        }
        for (int u = 0; b < n; b += T, u = (u + 1) & 3) s4[u] += __ldcg(src + (size_t)b * LSM_NSUM + q);
    }
    double v = (s4[0] + s4[1]) + (s4[2] + s4[3]);
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);  // within the T lanes of sum q
    if (q < NS && t == 0) dst[q] = v;
}

// lsm_sum_rows over float-float rows (the FP32 path mode).
template <int NS>
__device__ __forceinline__ void lsm_sum_rows_ff(const float2 *src, unsigned n, ff *dst) {
    constexpr int T = NS * 16 <= LSM_BLOCK ? 16 : 8;
    static_assert(NS * T <= LSM_BLOCK, "threads per sum");
    const int q = threadIdx.x / T, t = threadIdx.x % T;
    ff s4[4] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
    if (q < NS) {
        unsigned b = t;
        for (; b + 3 * T < n; b += 4 * T) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float2 v = __ldcg(src + (size_t)(b + T * u) * LSM_NSUM + q);
                s4[u] = ff_add(s4[u], ff{v.x, v.y});
            }
        }
        for (int u = 0; b < n; b += T, u = (u + 1) & 3) {
            const float2 v = __ldcg(src + (size_t)b * LSM_NSUM + q);
            s4[u] = ff_add(s4[u], ff{v.x, v.y});
        }
    }
    ff v = ff_add(ff_add(s4[0], s4[1]), ff_add(s4[2], s4[3]));
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) {
        const ff other{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        // the lower lane's value first, so both lanes of a pair compute the same sum
        v = (t & o) ? ff_add(other, v) : ff_add(v, other);
    }
    if (q < NS && t == 0) dst[q] = v;
}

// Waits until the published iteration count of a case reaches `want`
// (thread 0 polls, bounded); false when the wait gave up or another block
// reported an error. Called by the whole block.
__device__ __forceinline__ bool lsm_wait(const unsigned *ready, unsigned want, unsigned *err, int &flag,
                                         unsigned spin_limit) {
    __syncthreads();
    if (threadIdx.x == 0) {
        bool ok = true;
        unsigned n = 0;
        while (*(volatile const unsigned *)ready < want) {
            if (++n > spin_limit || *(volatile unsigned *)err != 0u) {
                ok = false;
                break;
            }
            __nanosleep(64);
        }
        if (!ok) atomicOr(err, 1u);
        __threadfence();
        flag = ok ? 1 : 0;
    }
    __syncthreads();
    return flag != 0;
}

// The paths of one tile read directly from global memory (see lsm_tile; the
// FP64 path mode); GEN: the payoff needs the interpreter.
template <class Real, int M, int B, bool GEN>
__device__ __forceinline__ void lsm_tile_paths(const LsmArgs &A, const KxProgram &P, const LsmPay<Real> &terms, int upd,
                                               int gram, bool fin, unsigned tile, bool have, const double (&cu)[M],
                                               const float (&cuf)[M], double disc_u, float disc_uf, double disc_g,
                                               float disc_gf, double (&acc)[M * (M + 1) / 2 + M + 1],
                                               float (&accf)[M * (M + 1) / 2 + M + 1]) {
    constexpr int NA = M * (M + 1) / 2;
    constexpr int NS = NA + M + 1;
    constexpr bool F32 = sizeof(Real) == 4;
    const int n_ex = A.n_ex;
    const uint64_t np = A.n_paths;
    const Real *S = reinterpret_cast<const Real *>(A.S);
    Real *V = reinterpret_cast<Real *>(A.value);
    const float inv_scale = A.inv_scale_f;
    const double d0 = A.disc[n_ex - 1];
    const Real *Su = S + (uint64_t)(upd >= 0 ? upd : n_ex - 1) * A.ld;
    const Real *Sg = S + (uint64_t)(gram >= 0 ? gram : 0) * A.ld;
    const uint64_t i0 = (uint64_t)tile * LSM_TILE + threadIdx.x;
    constexpr int CH = 4;  // paths whose loads are issued together
#pragma unroll 1
    for (int k0 = 0; k0 < LSM_PPT; k0 += CH) {
        Real su[CH], vv[CH], sg[CH];
#pragma unroll
        for (int k = 0; k < CH; ++k) {  // loads first (S is read-only here; V via L2)
            const uint64_t i = i0 + (uint64_t)(k0 + k) * LSM_BLOCK;
            const bool in = i < np;
            su[k] = in ? __ldg(Su + i) : Real(0);
            vv[k] = in && upd >= 0 ? __ldcg(V + i) : Real(0);
            sg[k] = in && gram >= 0 ? __ldg(Sg + i) : Real(0);
        }
#pragma unroll
        for (int k = 0; k < CH; ++k) {
            const uint64_t i = i0 + (uint64_t)(k0 + k) * LSM_BLOCK;
            if (i >= np) break;
            Real val;
            if (upd < 0) {
                val = lsm_pay_g<Real, GEN>(terms, P, su[k], n_ex);
            } else if (F32) {  // the decision in FP32 (FP64 only across threads)
                const float s = (float)su[k];
                const float pay = (float)lsm_pay_g<Real, GEN>(terms, P, (Real)s, upd + 1);
                const float discounted = (float)vv[k] * disc_uf;
                float nv = discounted;
                if (pay > 0.0f) {
                    float cont = discounted;
                    if (have) {
                        float phi[M];
                        lsm_basis_f32<M, B>(s * inv_scale, phi);
                        cont = 0.0f;
                        if (B == KX_LSM_MONOMIAL) {
#pragma unroll
                            for (int j = M - 1; j >= 0; --j) cont = cont * phi[1] + cuf[j];
                        } else {
#pragma unroll
                            for (int j = 0; j < M; ++j) cont += cuf[j] * phi[j];
                        }
                    }
                    nv = pay > cont ? pay : discounted;
                }
                val = (Real)nv;
            } else {
                const Real s = su[k];
                const Real pay = lsm_pay_g<Real, GEN>(terms, P, s, upd + 1);
                const double discounted = (double)vv[k] * disc_u;
                double nv = discounted;
                if (pay > Real(0)) {
                    double cont = discounted;
                    if (have) cont = lsm_continuation<M, B>(cu, (double)s, A.x_scale);
                    nv = (double)pay > cont ? (double)pay : discounted;
                }
                val = (Real)nv;
            }
            if (fin) {
                A.pv[i] = (double)val * d0;
                continue;
            }
            __stcg(V + i, val);
            if (lsm_pay_g<Real, GEN>(terms, P, sg[k], gram + 1) > Real(0)) {
                if (F32) {
                    const float yf = (float)val * disc_gf;
                    float pw[M];
                    lsm_basis_f32<M, B>((float)sg[k] * inv_scale, pw);
                    int q = 0;
#pragma unroll
                    for (int r = 0; r < M; ++r)
#pragma unroll
                        for (int c = r; c < M; ++c) accf[q++] += pw[r] * pw[c];
#pragma unroll
                    for (int r = 0; r < M; ++r) accf[NA + r] += pw[r] * yf;
                    accf[NS - 1] += 1.0f;
                } else {
                    const double x = (double)sg[k];
                    const double y = (double)val * disc_g;
                    double pw[M];
                    lsm_basis<M, B>(x, A.x_scale, pw);
                    int q = 0;
#pragma unroll
                    for (int r = 0; r < M; ++r)
#pragma unroll
                        for (int c = r; c < M; ++c) acc[q++] += __dmul_rn(pw[r], pw[c]);
#pragma unroll
                    for (int r = 0; r < M; ++r) acc[NA + r] += __dmul_rn(pw[r], y);
                    acc[NS - 1] += 1.0;
                }
            }
        }
    }
}

// Per-thread asynchronous 16-byte copies global -> shared (through L2, not
// L1: the values are written by other SMs between iterations).
__device__ __forceinline__ void lsm_cp16(void *smem_dst, const void *gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void lsm_cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void lsm_cp_wait_all_but() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void lsm_cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

constexpr int LSM_SUB = 4 * LSM_BLOCK;  // paths of an FP32 sub-chunk (4 per thread)
constexpr int LSM_NSTAGE = 4;           // sub-chunks in flight per thread
static_assert(LSM_TILE % LSM_SUB == 0, "whole sub-chunks per tile");

// One FP32 path at a decision date (and its regression date): the new
// realised value, and its terms of the normal equations added to accf.
template <int M, int B, bool GEN>
__device__ __forceinline__ float lsm_path_f32(const LsmPay<float> &terms, const KxProgram &P, int n_ex, int upd,
                                              int gram, bool fin, float su, float vv, float sg, bool have,
                                              const float (&cuf)[M], float disc_uf, float disc_gf, float inv_scale,
                                              float (&accf)[M * (M + 1) / 2 + M + 1]) {
    constexpr int NA = M * (M + 1) / 2;
    constexpr int NS = NA + M + 1;
    float val;
    if (upd < 0) {
        val = lsm_pay_g<float, GEN>(terms, P, su, n_ex);
    } else {  // the decision in FP32
        const float pay = lsm_pay_g<float, GEN>(terms, P, su, upd + 1);
        const float discounted = vv * disc_uf;
        float nv = discounted;
        if (pay > 0.0f) {
            float cont = discounted;
            if (have) {
                float phi[M];
                lsm_basis_f32<M, B>(su * inv_scale, phi);
                cont = 0.0f;
                if (B == KX_LSM_MONOMIAL) {
#pragma unroll
                    for (int j = M - 1; j >= 0; --j) cont = cont * phi[1] + cuf[j];
                } else {
#pragma unroll
                    for (int j = 0; j < M; ++j) cont += cuf[j] * phi[j];
                }
            }
            nv = pay > cont ? pay : discounted;
        }
        val = nv;
    }
    if (!fin && lsm_pay_g<float, GEN>(terms, P, sg, gram + 1) > 0.0f) {
        const float yf = val * disc_gf;
        float pw[M];
        lsm_basis_f32<M, B>(sg * inv_scale, pw);
        int q = 0;
#pragma unroll
        for (int r = 0; r < M; ++r)
#pragma unroll
            for (int c = r; c < M; ++c) accf[q++] += pw[r] * pw[c];
#pragma unroll
        for (int r = 0; r < M; ++r) accf[NA + r] += pw[r] * yf;
        accf[NS - 1] += 1.0f;
    }
    return val;
}

// The paths of one FP32 tile, streamed through a per-thread ring of
// LSM_NSTAGE sub-chunk slots in shared memory: thread j copies (asynchronous
// 16-byte copies through L2) and then reads only its own 4 consecutive paths
// of each sub-chunk, so no block barrier is needed while LSM_NSTAGE - 1
// sub-chunks stay in flight. ring: [LSM_NSTAGE][3][LSM_BLOCK] float4 (spots
// at the decision date, values, spots at the regression date). Rows of S are
// padded to 64 elements and the value array to 256 bytes, so a copy that
// starts before n_paths stays inside its allocation.
template <int M, int B, bool GEN>
__device__ __forceinline__ void lsm_tile_paths_ring(const LsmArgs &A, const KxProgram &P, const LsmPay<float> &terms,
                                                    int upd, int gram, bool fin, unsigned tile, float4 *ring, bool have,
                                                    const float (&cuf)[M], float disc_uf, float disc_gf,
                                                    float (&accf)[M * (M + 1) / 2 + M + 1]) {
    const int n_ex = A.n_ex;
    const uint64_t t0 = (uint64_t)tile * LSM_TILE;
    const uint64_t left = A.n_paths - t0;
    const uint64_t subs_left = (left + LSM_SUB - 1) / LSM_SUB;
    const int nsub = subs_left < (uint64_t)(LSM_TILE / LSM_SUB) ? (int)subs_left : LSM_TILE / LSM_SUB;
    const float *S = reinterpret_cast<const float *>(A.S);
    const float *Su = S + (uint64_t)(upd >= 0 ? upd : n_ex - 1) * A.ld + t0;
    const float *Sg = S + (uint64_t)(gram >= 0 ? gram : 0) * A.ld + t0;
    float *V = reinterpret_cast<float *>(A.value) + t0;
    double *pv = A.pv + t0;
    const float inv_scale = A.inv_scale_f;
    const double d0 = A.disc[n_ex - 1];
    const unsigned j = threadIdx.x;
    auto issue = [&](int sc) {
        const int slot = sc % LSM_NSTAGE;
        const uint64_t e = (uint64_t)sc * LSM_SUB + 4u * j;
        if (e < left) {
            lsm_cp16(ring + (slot * 3 + 0) * LSM_BLOCK + j, Su + e);
            if (upd >= 0) lsm_cp16(ring + (slot * 3 + 1) * LSM_BLOCK + j, V + e);
            if (gram >= 0) lsm_cp16(ring + (slot * 3 + 2) * LSM_BLOCK + j, Sg + e);
        }
        lsm_cp_commit();
    };
#pragma unroll 1
    for (int sc = 0; sc < LSM_NSTAGE - 1; ++sc) {
        if (sc < nsub) issue(sc);
        else lsm_cp_commit();
    }
#pragma unroll 1
    for (int sc = 0; sc < nsub; ++sc) {
        if (sc + LSM_NSTAGE - 1 < nsub) issue(sc + LSM_NSTAGE - 1);
        else lsm_cp_commit();
        lsm_cp_wait_all_but<LSM_NSTAGE - 1>();  // this thread's copies of sub-chunk sc have landed
        const uint64_t e = (uint64_t)sc * LSM_SUB + 4u * j;
        if (e >= left) continue;
        const int slot = sc % LSM_NSTAGE;
        const float4 su = ring[(slot * 3 + 0) * LSM_BLOCK + j];
        const float4 vv = upd >= 0 ? ring[(slot * 3 + 1) * LSM_BLOCK + j] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 sg = gram >= 0 ? ring[(slot * 3 + 2) * LSM_BLOCK + j] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int nq = left - e >= 4 ? 4 : (int)(left - e);
        float v[4];
        v[0] = lsm_path_f32<M, B, GEN>(terms, P, n_ex, upd, gram, fin, su.x, vv.x, sg.x, have, cuf, disc_uf, disc_gf,
                                       inv_scale, accf);
        if (nq > 1)
            v[1] = lsm_path_f32<M, B, GEN>(terms, P, n_ex, upd, gram, fin, su.y, vv.y, sg.y, have, cuf, disc_uf,
                                           disc_gf, inv_scale, accf);
        if (nq > 2)
            v[2] = lsm_path_f32<M, B, GEN>(terms, P, n_ex, upd, gram, fin, su.z, vv.z, sg.z, have, cuf, disc_uf,
                                           disc_gf, inv_scale, accf);
        if (nq > 3)
            v[3] = lsm_path_f32<M, B, GEN>(terms, P, n_ex, upd, gram, fin, su.w, vv.w, sg.w, have, cuf, disc_uf,
                                           disc_gf, inv_scale, accf);
        if (fin) {
            for (int q = 0; q < nq; ++q) pv[e + q] = (double)v[q] * d0;
        } else if (nq == 4) {
            __stcg(reinterpret_cast<float4 *>(V + e), make_float4(v[0], v[1], v[2], v[3]));
        } else {
            for (int q = 0; q < nq; ++q) __stcg(V + e + q, v[q]);
        }
    }
}

// A tile block's walk over its items: iterations in order, in each the cases
// still active in case order, and of each case the tiles w = blk, blk + nb,
// ... of the iteration's item numbering (the tiles of the active cases, in
// case order).
struct LsmCursor {
    int it, c;
    unsigned base, w;
};
__device__ __forceinline__ bool lsm_advance(const LsmArgs *cases, int n_cases, int max_ex, unsigned nb, unsigned blk,
                                            LsmCursor &k, bool first) {
    if (!first) {
        k.w += nb;
        if (k.w < k.base + cases[k.c].n_tiles) return true;
        k.base += cases[k.c].n_tiles;
        ++k.c;
    }
    for (; k.it < max_ex; ++k.it, k.c = 0, k.base = 0) {
        for (; k.c < n_cases; ++k.c) {
            const LsmArgs &A = cases[k.c];
            if (k.it >= A.n_ex || A.n_tiles == 0) continue;
            k.w = k.base + (blk + nb - k.base % nb) % nb;
            if (k.w < k.base + A.n_tiles) return true;
            k.base += A.n_tiles;
        }
    }
    return false;
}

// One tile of one backward iteration `it` of a case: apply the decision of
// date upd = n_ex - 1 - it to the tile's realised values (it = 0: set them to
// the payoff at the last date), accumulate the normal equations of date
// gram = upd - 1 over the tile's in-the-money paths (lsm.rs:259-288), and, in
// the last iteration, discount the values to t = 0 (lsm.rs:226). The tile's
// sums go to its slot and the tile is counted; the coordinator block solves.
template <class Real, int M, int B, bool GEN>
__device__ void lsm_tile(const LsmArgs &A, int it, unsigned tile, double *red, float4 *ring) {
    constexpr int NA = M * (M + 1) / 2;
    constexpr int NS = NA + M + 1;  // A upper triangle, A^T y, ITM count
    static_assert(NS <= LSM_NSUM, "partial stride");
    constexpr bool F32 = sizeof(Real) == 4;
    const int n_ex = A.n_ex;
    const int upd = it == 0 ? -1 : n_ex - 1 - it;
    const int gram = n_ex - 2 - it;
    const bool fin = it == n_ex - 1;
    const KxProgram &P = *A.P;
    double acc[NS];
    float accf[NS];
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        acc[q] = 0.0;
        accf[q] = 0.0f;
    }
    double cu[M];
    float cuf[M];
    bool have = false;
    if (upd >= 0) {
        const float *cf = reinterpret_cast<const float *>(A.coef + upd * LSM_COEF + 8);
        have = __ldcg(cf + 7) != 0.0f;
#pragma unroll
        for (int j = 0; j < M; ++j) {
            if (!F32) cu[j] = __ldcg(A.coef + upd * LSM_COEF + j);
            cuf[j] = __ldcg(cf + j);
        }
    }
    const LsmPay<Real> terms = lsm_pay_terms<Real>(A.pay);
    const double disc_u = !F32 && upd >= 0 ? A.disc[upd] : 0.0;
    const float disc_uf = upd >= 0 ? A.disc_f[upd] : 0.0f;
    const double disc_g = !F32 && gram >= 0 ? A.disc[gram] : 0.0;
    const float disc_gf = gram >= 0 ? A.disc_f[gram] : 0.0f;
    if constexpr (F32)
        lsm_tile_paths_ring<M, B, GEN>(A, P, terms, upd, gram, fin, tile, ring, have, cuf, disc_uf, disc_gf, accf);
    else
        lsm_tile_paths<Real, M, B, GEN>(A, P, terms, upd, gram, fin, tile, have, cu, cuf, disc_u, disc_uf, disc_g,
                                        disc_gf, acc, accf);
    if (gram < 0) return;
    // the tile's partial sums (FP32 paths: float-float, FP64 paths: FP64)
    if (F32) {
        ff *out = reinterpret_cast<ff *>(red + LSM_RED_OUT);
        block_sums_ff(accf, NS, red, out);
        if (threadIdx.x < NS)
            __stcg(reinterpret_cast<float2 *>(A.partial) + (size_t)tile * LSM_NSUM + threadIdx.x,
                   make_float2(out[threadIdx.x].hi, out[threadIdx.x].lo));
    } else {
        block_sums(acc, NS, red);
        if (threadIdx.x < NS) __stcg(A.partial + (size_t)tile * LSM_NSUM + threadIdx.x, red[LSM_RED_OUT + threadIdx.x]);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(A.sync + 1, 1u);  // the coordinator counts the tiles
}

// The regression of one case and iteration, once all its tiles arrived: the
// tiles' sums added in tile order, the m x m system solved (FP64 paths:
// exactly as numerics::solve_linear, numerics.rs:190-236, Gauss with partial
// pivoting, a pivot below 1e-12 gives zero coefficients; FP32 paths: the same
// in float-float), the coefficients of date gram published. Run by the
// coordinator block, always on the same SM, so this long straight-line code
// stays in its instruction cache (run once per date on whichever SM finished
// last, it was bound by instruction fetch).
template <class Real, int M>
__device__ void lsm_solve_case(const LsmArgs &A, int it, double *red) {
    constexpr int NA = M * (M + 1) / 2;
    constexpr int NS = NA + M + 1;
    constexpr bool F32 = sizeof(Real) == 4;
    const int gram = A.n_ex - 2 - it;
    __threadfence();
    if (F32) lsm_sum_rows_ff<NS>(reinterpret_cast<const float2 *>(A.partial), A.n_tiles, reinterpret_cast<ff *>(red));
    else lsm_sum_rows<NS>(A.partial, A.n_tiles, red);
    __syncthreads();
    if (threadIdx.x < 32) {  // the solve on warp 0
        float *cf = reinterpret_cast<float *>(A.coef + gram * LSM_COEF + 8);
        if (F32) {
            const ff *rf = reinterpret_cast<const ff *>(red);
            const bool fit = rf[NS - 1].hi >= (float)M;  // lsm.rs:190-194
            ff x[LSM_MAXM];
            if (fit) solve_gauss_warp_ff<M>(rf, NA, x);
            if (threadIdx.x == 0) {
                for (int j = 0; j < M; ++j) cf[j] = fit ? x[j].hi : 0.0f;  // hi = the float nearest hi + lo
                cf[7] = fit ? 1.0f : 0.0f;
            }
        } else {
            const bool fit = red[NS - 1] >= (double)M;  // lsm.rs:190-194
            double x[LSM_MAXM];
            if (fit) solve_gauss_warp<M>(red, NA, x);
            if (threadIdx.x == 0) {
                for (int j = 0; j < M; ++j) {
                    A.coef[gram * LSM_COEF + j] = fit ? x[j] : 0.0;
                    cf[j] = fit ? (float)x[j] : 0.0f;
                }
                cf[7] = fit ? 1.0f : 0.0f;
            }
        }
        if (threadIdx.x == 0) {
            A.sync[1] = 0u;
            __threadfence();
            atomicExch(A.sync, (unsigned)it + 1u);  // publish: iteration `it` is solved
        }
    }
    __syncthreads();
}

// Coordinator block k of n_coord: polls the tile counts of its cases c = k,
// k + n_coord, ... (one thread per case, so one round trip covers them) and
// runs lsm_solve_case for every case whose iteration is complete, the lowest
// case first. Each case has n_ex - 1 regressions (iterations 0 .. n_ex - 2).
// A poll that sees no progress for spin_limit rounds gives up and sets the
// error word.
template <class Real, int M>
__device__ void lsm_coordinator(const LsmArgs *cases, int n_cases, int k, int n_coord, unsigned *err, double *red,
                                int *next, int &ready_c, unsigned spin_limit) {
    for (int c = threadIdx.x; c < n_cases; c += blockDim.x) next[c] = 0;
    __syncthreads();
    unsigned idle = 0;
    for (;;) {
        // one thread per case: the first case whose pending iteration is complete
        if (threadIdx.x == 0) ready_c = n_cases;
        __syncthreads();
        bool open = false;
        for (int c = k + threadIdx.x * n_coord; c < n_cases; c += blockDim.x * n_coord) {
            const LsmArgs &A = cases[c];
            if (A.n_tiles == 0 || next[c] >= A.n_ex - 1) continue;
            open = true;
            if (*(volatile const unsigned *)(A.sync + 1) == A.n_tiles) atomicMin(&ready_c, c);
        }
        const bool any_open = __syncthreads_or(open);
        if (!any_open) return;
        const int c = ready_c;
        if (c < n_cases) {
            idle = 0;
            lsm_solve_case<Real, M>(cases[c], next[c], red);
            if (threadIdx.x == 0) ++next[c];
            __syncthreads();
        } else {
            if (++idle > spin_limit || *(volatile unsigned *)err != 0u) {
                if (threadIdx.x == 0) atomicOr(err, 1u);
                return;
            }
            __nanosleep(32);
        }
    }
}

// The backward induction of every case in one cooperative launch (all
// blocks resident). Iteration `it` of case c covers its tiles; the items of
// an iteration (the tiles of the cases still active, in case order) are
// dealt round-robin to the tile blocks; the last n_coord blocks coordinate
// (sums and solves, case c on coordinator c % n_coord). A tile block waits only for the solve of the previous iteration
// of the case whose tile it takes next, so different cases' dates overlap and
// no launch ends between dates.
template <class Real, int M, int B, bool GEN>
__global__ void __launch_bounds__(LSM_BLOCK, sizeof(Real) == 4 ? 4 : 2)
    k_lsm_backward(const LsmArgs *__restrict__ cases, int n_cases, int max_ex, int n_coord, unsigned *err,
                   unsigned spin_limit) {
    __shared__ double red[LSM_RED_OUT + 32];
    __shared__ int flag;
    const unsigned n_tile_blocks = gridDim.x - (unsigned)n_coord;
    if (blockIdx.x >= n_tile_blocks) {  // the coordinators: the regression solves
        __shared__ int next[LSM_MAX_CASES];
        lsm_coordinator<Real, M>(cases, n_cases, (int)(blockIdx.x - n_tile_blocks), n_coord, err, red, next, flag,
                                 spin_limit);
        return;
    }
    extern __shared__ __align__(16) float4 lsm_ring[];  // FP32: [LSM_NSTAGE][3][LSM_BLOCK]
    LsmCursor cur{0, 0, 0u, 0u};
    bool more = lsm_advance(cases, n_cases, max_ex, n_tile_blocks, blockIdx.x, cur, true);
    int seen_c = -1, seen_it = -1;  // the last (case, iteration) whose solve this block saw published
    while (more) {
        const LsmArgs &A = cases[cur.c];
        if (cur.it > 0 && (cur.c != seen_c || cur.it != seen_it)) {
            if (!lsm_wait(A.sync, (unsigned)cur.it, err, flag, spin_limit)) break;
            seen_c = cur.c;
            seen_it = cur.it;
        }
        lsm_tile<Real, M, B, GEN>(A, cur.it, cur.w - cur.base, red, lsm_ring);
        more = lsm_advance(cases, n_cases, max_ex, n_tile_blocks, blockIdx.x, cur, false);
    }
    lsm_cp_wait_all();
}

// GEN: some payoff of the call needs the interpreter (a kernel without it has
// no call and keeps its state in registers).
template <class Real, int M>
static const void *backward_kernel_m(int basis, bool gen) {
    if (gen)
        return basis == KX_LSM_LAGUERRE ? (const void *)k_lsm_backward<Real, M, KX_LSM_LAGUERRE, true>
                                        : (const void *)k_lsm_backward<Real, M, KX_LSM_MONOMIAL, true>;
    return basis == KX_LSM_LAGUERRE ? (const void *)k_lsm_backward<Real, M, KX_LSM_LAGUERRE, false>
                                    : (const void *)k_lsm_backward<Real, M, KX_LSM_MONOMIAL, false>;
}

template <class Real>
static const void *backward_kernel(int m, int basis, bool gen) {
    switch (m) {
    case 2: return backward_kernel_m<Real, 2>(basis, gen);
    case 3: return backward_kernel_m<Real, 3>(basis, gen);
    case 4: return backward_kernel_m<Real, 4>(basis, gen);
    case 5: return backward_kernel_m<Real, 5>(basis, gen);
    default: return backward_kernel_m<Real, 6>(basis, gen);
    }
}

struct LsmCase {
    KxProgram P;
    std::vector<unsigned char> steps;  // StepRec<Real> of [0, dates...]
    std::vector<double> disc;
    LsmArgs a;                         // device pointers filled by the caller
    Model m;
    uint64_t np = 0;
    int n_ex = 0;
};

static LsmCase lsm_case(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg, const double *dates,
                        size_t n_dates, int32_t n_basis, int32_t basis) {
    if (basis != KX_LSM_MONOMIAL && basis != KX_LSM_LAGUERRE) raise(KX_INVALID_ARGUMENT, "unknown LSM basis");
    const Program &p = program_of(prog);
    LsmCase L;
    L.m = model_from_c(model);
    if (!cfg) raise(KX_INVALID_ARGUMENT, "NULL argument");
    if (cfg->flags != 0 || (cfg->rng != KX_RNG_PHILOX && cfg->rng != KX_RNG_SHARED_DRAWS) ||
        (cfg->precision != KX_PREC_FP32 && cfg->precision != KX_PREC_FP64))
        raise(KX_INVALID_ARGUMENT, "bad config");
    if (n_dates == 0 || !dates) raise(KX_MALFORMED_CONTRACT, "LSM: at least one exercise date required");
    for (size_t i = 1; i < n_dates; ++i)
        if (!(dates[i] > dates[i - 1])) raise(KX_MALFORMED_CONTRACT, "LSM: exercise dates must increase and be > 0");
    if (!(dates[0] > 0.0)) raise(KX_MALFORMED_CONTRACT, "LSM: exercise dates must increase and be > 0");
    if (n_basis < 2) raise(KX_MALFORMED_CONTRACT, "LSM: n_basis >= 2 required");
    if (n_basis > LSM_MAXM) raise(KX_UNSUPPORTED, "LSM: n_basis above 6 is not supported on the device");
    const KxProgram &Lw = p.low.prog;
    if (Lw.n_trig != 0 || Lw.n_acc != 0)
        raise(KX_UNSUPPORTED, "LSM payoff must be an immediate function of the spot "
                              "(no when/until/anytime, averages or running extrema)");
    validate_model(L.m);
    std::vector<double> grid{0.0};
    grid.insert(grid.end(), dates, dates + n_dates);
    validate_grid(grid);
    const bool f64 = cfg->precision == KX_PREC_FP64;
    L.np = cfg->n_paths;
    StepTables tab;
    bind(p.low, grid, L.m, cfg->rate, L.P, tab);
    L.n_ex = (int)n_dates;
    L.disc.resize(L.n_ex);
    for (int d = 0; d + 1 < L.n_ex; ++d) L.disc[d] = std::exp(-cfg->rate * (dates[d + 1] - dates[d]));  // lsm.rs:176
    L.disc[L.n_ex - 1] = std::exp(-cfg->rate * dates[0]);                                               // lsm.rs:226
    {  // the FP32 copies follow the doubles in the same table
        const size_t nd = (size_t)L.n_ex;
        L.disc.resize(nd + (nd + 1) / 2);
        float *f = reinterpret_cast<float *>(L.disc.data() + nd);
        for (size_t d = 0; d < nd; ++d) f[d] = (float)L.disc[d];
    }
    L.steps.resize(grid.size() * (f64 ? sizeof(StepRec<double>) : sizeof(StepRec<float>)));
    for (size_t k = 0; k < grid.size(); ++k) {
        if (f64) reinterpret_cast<StepRec<double> *>(L.steps.data())[k] = {tab.c0[k], tab.c1[k], 0u, 0u};
        else reinterpret_cast<StepRec<float> *>(L.steps.data())[k] = {(float)tab.c0[k], (float)tab.c1[k], 0u, 0u};
    }
    LsmArgs &a = L.a;
    a = LsmArgs{};
    a.n_times = (int)grid.size();
    a.n_ex = L.n_ex;
    a.n_paths = L.np;
    a.seed = cfg->seed;
    a.model = L.m.kind;
    a.scheme = L.m.scheme;
    a.s0 = L.m.s0;
    a.v0 = L.m.v0; a.kappa = L.m.kappa; a.theta = L.m.theta; a.sigma_v = L.m.sigma_v; a.rho = L.m.rho;
    a.rho_perp = std::sqrt(std::max(1.0 - L.m.rho * L.m.rho, 0.0));
    a.r = L.m.r;
    a.x_scale = L.m.s0;
    a.s0_f = (float)a.s0; a.v0_f = (float)std::max(a.v0, 0.0); a.kappa_f = (float)a.kappa;
    a.theta_f = (float)a.theta; a.sigma_v_f = (float)a.sigma_v; a.rho_f = (float)a.rho;
    a.rho_perp_f = (float)a.rho_perp; a.r_f = (float)a.r;
    a.inv_scale_f = (float)(1.0 / a.x_scale);
    a.pay = lsm_pay_tab(L.P);
    return L;
}


// Device memory of a set of cases, carved from one arena: per case its
// program, steps, discounts, stored paths, values, per-path results, tile and
// coefficients and synchronisation words; then the case
// table and the error word.
static size_t lsm_al(size_t x) { return (x + 255) & ~size_t(255); }
static uint64_t lsm_ld(uint64_t n_paths) { return (n_paths + 63) & ~uint64_t(63); }

static size_t lsm_case_bytes(const LsmCase &L, size_t rs) {
    const unsigned nt = lsm_tiles(L.np);
    return lsm_al(sizeof(KxProgram)) + lsm_al(L.steps.size()) + lsm_al(L.disc.size() * sizeof(double)) +
           lsm_al(std::max<uint64_t>(1, lsm_ld(L.np) * L.n_ex) * rs) + lsm_al(std::max<uint64_t>(1, L.np) * rs) +
           lsm_al(std::max<uint64_t>(1, L.np) * sizeof(double)) + lsm_al((size_t)std::max(1u, nt) * LSM_NSUM * 8) +
           lsm_al((size_t)L.n_ex * LSM_COEF * sizeof(double)) + lsm_al(2 * sizeof(unsigned));
}

// Prices the cases (all of one precision): uploads, forward simulations, the
// cooperative backward launch, per-path statistics.
static void lsm_run(Ctx &c, std::vector<LsmCase> &cs, bool f64, int n_basis, int basis, kx_price_result *out,
                    double *const *per_path = nullptr) {
    const size_t n = cs.size();
    const size_t rs = f64 ? 8 : 4;
    std::vector<size_t> off(n + 1, 0);
    int max_ex = 0;
    uint64_t tot_tiles = 0;
    for (size_t i = 0; i < n; ++i) {
        off[i + 1] = off[i] + lsm_case_bytes(cs[i], rs);
        max_ex = std::max(max_ex, cs[i].n_ex);
        tot_tiles += lsm_tiles(cs[i].np);
    }
    const size_t off_cases = off[n], off_err = lsm_al(off_cases + n * sizeof(LsmArgs));
    c.lsm_paths.ensure(off_err + 256);
    unsigned char *base = c.lsm_paths.as<unsigned char>();
    std::vector<LsmArgs> args(n);
    std::vector<StatsJob> sj(n);
    for (size_t i = 0; i < n; ++i) {
        LsmCase &L = cs[i];
        const unsigned nt = lsm_tiles(L.np);
        unsigned char *q = base + off[i];
        auto take = [&](size_t bytes) {
            unsigned char *r = q;
            q += lsm_al(bytes);
            return r;
        };
        LsmArgs &a = L.a;
        a.P = reinterpret_cast<const KxProgram *>(take(sizeof(KxProgram)));
        a.steps = take(L.steps.size());
        a.disc = reinterpret_cast<const double *>(take(L.disc.size() * sizeof(double)));
        a.disc_f = reinterpret_cast<const float *>(a.disc + L.n_ex);
        a.S = take(std::max<uint64_t>(1, lsm_ld(L.np) * L.n_ex) * rs);
        a.ld = lsm_ld(L.np);
        a.value = take(std::max<uint64_t>(1, L.np) * rs);
        a.pv = reinterpret_cast<double *>(take(std::max<uint64_t>(1, L.np) * sizeof(double)));
        a.partial = reinterpret_cast<double *>(take((size_t)std::max(1u, nt) * LSM_NSUM * 8));
        a.coef = reinterpret_cast<double *>(take((size_t)L.n_ex * LSM_COEF * sizeof(double)));
        a.sync = reinterpret_cast<unsigned *>(take(2 * sizeof(unsigned)));
        a.n_tiles = nt;
        KX_CUDA(cudaMemcpyAsync((void *)a.P, &L.P, sizeof(KxProgram), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync((void *)a.steps, L.steps.data(), L.steps.size(), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync((void *)a.disc, L.disc.data(), L.disc.size() * sizeof(double), cudaMemcpyHostToDevice,
                                c.stream));
        KX_CUDA(cudaMemsetAsync(a.sync, 0, 2 * sizeof(unsigned), c.stream));
        c.last.h2d_bytes += sizeof(KxProgram) + L.steps.size() + L.disc.size() * sizeof(double);
        args[i] = a;
        sj[i].begin = (uint64_t)(reinterpret_cast<unsigned char *>(a.pv) - base) / sizeof(double);
        sj[i].n = L.np;
        c.last.path_steps += L.np * (uint64_t)L.n_ex;
    }
    c.last.steps_simulated = c.last.path_steps;
    LsmArgs *cases_dev = reinterpret_cast<LsmArgs *>(base + off_cases);
    unsigned *err = reinterpret_cast<unsigned *>(base + off_err);
    KX_CUDA(cudaMemcpyAsync(cases_dev, args.data(), n * sizeof(LsmArgs), cudaMemcpyHostToDevice, c.stream));
    KX_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), c.stream));
    c.last.h2d_bytes += n * sizeof(LsmArgs);
    if (tot_tiles > 0) {
        const int fblocks = c.sm_count * 4;
        KX_CUDA(cudaEventRecord(c.ev0, c.stream));
        for (auto &L : cs) {  // forward simulations (each writes its own S)
            if (L.np == 0) continue;
            if (f64) {
                if (L.m.kind == KX_MODEL_GBM) k_lsm_forward<double, KX_MODEL_GBM><<<fblocks, LSM_BLOCK, 0, c.stream>>>(L.a);
                else k_lsm_forward<double, KX_MODEL_HESTON><<<fblocks, LSM_BLOCK, 0, c.stream>>>(L.a);
            } else {  // four paths per thread, one 16-byte store per date; one group per thread
                const uint64_t groups = (L.np + 3) / 4;
                const unsigned gb = (unsigned)std::min<uint64_t>((groups + LSM_BLOCK - 1) / LSM_BLOCK,
                                                                 (uint64_t)c.sm_count * 64);
                if (L.m.kind == KX_MODEL_GBM) k_lsm_forward4<KX_MODEL_GBM><<<gb, LSM_BLOCK, 0, c.stream>>>(L.a);
                else k_lsm_forward4<KX_MODEL_HESTON><<<gb, LSM_BLOCK, 0, c.stream>>>(L.a);
            }
            KX_CUDA(cudaGetLastError());
            c.last.kernel_launches++;
        }
        bool gen = false;
        for (auto &L : cs) gen = gen || !L.a.pay.ok;
        const void *kfn = f64 ? backward_kernel<double>(n_basis, basis, gen) : backward_kernel<float>(n_basis, basis, gen);
        // FP32: the per-thread staging rings in dynamic shared memory
        const size_t dyn = f64 ? 0 : (size_t)LSM_NSTAGE * 3 * LSM_BLOCK * sizeof(float4);
        KX_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
        KX_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared));
        int per_sm = 0;
        KX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, LSM_BLOCK, dyn));
        if (per_sm < 1) raise(KX_CUDA_ERROR, "LSM backward kernel cannot be resident");
        // every block resident (the blocks wait on one another): at most one tile block per tile,
        // plus the coordinators (one per case up to LSM_MAX_COORD)
        int n_coord = (int)std::min<size_t>(n, LSM_MAX_COORD);
        const uint64_t cap = (uint64_t)per_sm * c.sm_count;
        if (cap < (uint64_t)n_coord + 1) n_coord = (int)std::max<uint64_t>(1, cap / 2);
        const unsigned grid = (unsigned)std::min<uint64_t>(cap, tot_tiles + n_coord);
        int n_cases = (int)n;
        // every wait of the launch gives up after spin_limit polls; a test sets a tiny limit through
        // KX_LSM_SPIN_LIMIT to make a wait run out (the call then fails with KX_DEVICE_TIMEOUT)
        unsigned spin_limit = LSM_SPIN_LIMIT;
        if (const char *e = getenv("KX_LSM_SPIN_LIMIT")) spin_limit = (unsigned)strtoul(e, nullptr, 10);
        void *kargs[] = {(void *)&cases_dev, (void *)&n_cases, (void *)&max_ex, (void *)&n_coord, (void *)&err,
                         (void *)&spin_limit};
        KX_CUDA(cudaLaunchCooperativeKernel(kfn, dim3(grid), dim3(LSM_BLOCK), kargs, dyn, c.stream));
        c.last.kernel_launches++;
        KX_CUDA(cudaEventRecord(c.ev1, c.stream));
        KX_CUDA(cudaEventSynchronize(c.ev1));
        float ms = 0.f;
        KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        c.last.kernel_ms += ms;
        unsigned herr = 0;
        KX_CUDA(cudaMemcpy(&herr, err, sizeof herr, cudaMemcpyDeviceToHost));
        if (herr) raise(KX_DEVICE_TIMEOUT, "LSM backward induction: a wait for a regression solve gave up");
    }
    auto st = device_stats(c, reinterpret_cast<const double *>(base), 0, sj);
    for (size_t i = 0; i < n; ++i) out[i] = finish(st[i]);
    if (per_path)
        for (size_t i = 0; i < n; ++i)
            if (per_path[i] && cs[i].np) {
                KX_CUDA(cudaMemcpy(per_path[i], cs[i].a.pv, cs[i].np * sizeof(double), cudaMemcpyDeviceToHost));
                c.last.d2h_bytes += cs[i].np * sizeof(double);
            }
}

}  // namespace kx

using namespace kx;

extern "C" kx_status kx_price_american_lsm_paths(const kx_program *prog, const kx_model *model,
                                                 const kx_mc_config *cfg, const double *dates, size_t n_dates,
                                                 int32_t n_basis, int32_t basis, kx_price_result *out,
                                                 double *per_path_pv) {
    return guarded([&] {
        if (!out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        std::vector<LsmCase> cs;
        cs.push_back(lsm_case(prog, model, cfg, dates, n_dates, n_basis, basis));
        LsmCase &L = cs[0];
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        if (cfg->rng == KX_RNG_SHARED_DRAWS) {
            DrawStore &ds = c.draws;
            if (!ds.set) raise(KX_INVALID_ARGUMENT, "no shared draws registered");
            if (ds.n_paths < L.np || ds.dpp < (uint64_t)L.n_ex * L.m.draws_per_step())
                raise(KX_INVALID_ARGUMENT, "shared draws too small for this simulation");
            L.a.z64 = ds.is64 ? ds.z64.as<double>() : nullptr;
            L.a.z32 = ds.is64 ? nullptr : ds.z32.as<float>();
            L.a.z_dpp = ds.dpp;
        }
        lsm_run(c, cs, cfg->precision == KX_PREC_FP64, n_basis, basis, out, &per_path_pv);
        c.last.total_ms += now_ms();
    });
}

extern "C" kx_status kx_price_american_lsm_basis(const kx_program *prog, const kx_model *model,
                                                 const kx_mc_config *cfg, const double *dates, size_t n_dates,
                                                 int32_t n_basis, int32_t basis, kx_price_result *out) {
    return kx_price_american_lsm_paths(prog, model, cfg, dates, n_dates, n_basis, basis, out, nullptr);
}

extern "C" kx_status kx_price_american_lsm(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg,
                                           const double *dates, size_t n_dates, int32_t n_basis,
                                           kx_price_result *out) {
    return kx_price_american_lsm_basis(prog, model, cfg, dates, n_dates, n_basis, KX_LSM_MONOMIAL, out);
}

extern "C" kx_status kx_price_american_lsm_batch(size_t n, const kx_program *const *progs, const kx_model *models,
                                                 const kx_mc_config *cfgs, const double *const *dates,
                                                 const size_t *n_dates, int32_t n_basis, int32_t basis,
                                                 kx_price_result *out) {
    return guarded([&] {
        if (n == 0) return;
        if (!progs || !models || !cfgs || !dates || !n_dates || !out) raise(KX_INVALID_ARGUMENT, "NULL array");
        if (n > (size_t)LSM_MAX_CASES) raise(KX_INVALID_ARGUMENT, "an LSM batch holds at most 1024 cases");
        std::vector<LsmCase> cs;
        for (size_t i = 0; i < n; ++i) {
            cs.push_back(lsm_case(progs[i], &models[i], &cfgs[i], dates[i], n_dates[i], n_basis, basis));
            if (cfgs[i].rng != KX_RNG_PHILOX) raise(KX_INVALID_ARGUMENT, "an LSM batch draws from Philox");
            if (cfgs[i].precision != cfgs[0].precision) raise(KX_INVALID_ARGUMENT, "an LSM batch has one precision");
        }
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        lsm_run(c, cs, cfgs[0].precision == KX_PREC_FP64, n_basis, basis, out);
        c.last.total_ms += now_ms();
    });
}
