// lsm.cu — Longstaff-Schwartz American pricing on the GPU
// (price_american_lsm / backward_induction, src/lsm.rs:80-229).
//
//  1. k_lsm_forward simulates every path on the grid [0, dates...] (the same
//     Philox counters as the European kernels, so the same paths) and stores
//     S at each exercise date in HBM, date-major: S[d * n_paths + i], so that
//     consecutive threads write and read consecutive addresses.
//  2. One k_lsm_step launch per exercise date, walking backwards. Launch d
//     applies the exercise decision of date d to every path's realised value
//     (lsm.rs:196-222) and, in the same pass, accumulates the FP64 normal
//     equations A^T A, A^T y of date d-1 over the in-the-money paths
//     (lsm.rs:259-288: monomial basis 1, S, ..., S^(m-1)). Each block writes
//     its partial sums to a fixed slot; the last block to finish adds them in
//     block order (deterministic) and solves the m x m system by Gauss
//     elimination with partial pivoting, exactly as numerics::solve_linear
//     (numerics.rs:190-236): a pivot below 1e-12 gives zero coefficients.
//  3. k_lsm_final discounts the values to t = 0; the per-path values then go
//     through the same deterministic statistics as every price.
// The launches are queued back to back with no host synchronisation.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "device_common.cuh"
#include "engine.hpp"

namespace kx {

constexpr int LSM_BLOCK = 256;
constexpr int LSM_MAXM = 6;
constexpr int LSM_COEF = 8;  // coef[d * LSM_COEF + j], j < m; [7] = have-fit flag

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
    const double *z64;
    const float *z32;
    uint64_t z_dpp;
    void *S;           // Real[n_ex][n_paths]
    void *value;       // Real[n_paths]: realised value at the current date
    double *pv;        // final per-path values
    double *partial;   // [gridDim][nsum]
    double *coef;      // [n_ex][LSM_COEF]
    unsigned *ticket;
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

template <class Real>
__device__ __forceinline__ LsmPay<Real> lsm_pay_terms(const KxProgram &P) {
    LsmPay<Real> t;
    t.ok = P.n_leaf <= 4;
    t.n = 0;
    for (int j = 0; j < P.n_leaf && t.ok; ++j) {
        const KxLeaf &F = P.leaf[j];
        if (F.kind != AK_CONST && !F.fast) t.ok = false;
        t.kind[t.n] = F.kind == AK_CONST ? (uint8_t)FA_NONE : F.fast;
        t.k[t.n] = F.kind == AK_CONST ? Real(0) : (Real)P.cpool[F.fast_k];
        t.sign[t.n] = (Real)F.sign;
        ++t.n;
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

template <class Real, int MODEL>
__global__ void __launch_bounds__(LSM_BLOCK) k_lsm_forward(const LsmArgs A) {
    constexpr int DRAWS = MODEL == KX_MODEL_GBM ? 1 : 2;
    const StepRec<Real> *R = reinterpret_cast<const StepRec<Real> *>(A.steps);
    Real *S = reinterpret_cast<Real *>(A.S);
    const Real s0 = (Real)A.s0, r = (Real)A.r, kap = (Real)A.kappa, th = (Real)A.theta, sv = (Real)A.sigma_v,
               rho = (Real)A.rho, rp = (Real)A.rho_perp;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < A.n_paths;
         i += (uint64_t)gridDim.x * blockDim.x) {
        Real y = Real(0), v = (Real)fmax(A.v0, 0.0);
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
            S[(uint64_t)(k - 1) * A.n_paths + i] = s0 * fast_exp<Real>(y);
        }
    }
}

// Block-wide sum of `n` doubles per thread into red[0..n) (fixed order).
__device__ void block_sums(double *vals, int n, double *red) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int q = 0; q < n; ++q) {
        double v = vals[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0) red[q * 32 + w] = v;
    }
    __syncthreads();
    if (threadIdx.x < n) {
        double t = 0.0;
        for (int j = 0; j < nw; ++j) t += red[threadIdx.x * 32 + j];
        red[32 * 64 + threadIdx.x] = t;
    }
    __syncthreads();
}

// The same for FP32 partial sums: the warp adds its 32 lanes in FP32, the
// warps' totals are added in FP64 (fixed order).
__device__ void block_sums_f32(const float *vals, int n, double *red) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int q = 0; q < n; ++q) {
        float v = vals[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0) red[q * 32 + w] = (double)v;
    }
    __syncthreads();
    if (threadIdx.x < n) {
        double t = 0.0;
        for (int j = 0; j < nw; ++j) t += red[threadIdx.x * 32 + j];
        red[32 * 64 + threadIdx.x] = t;
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

// One backward launch: update the values with the decision of date `upd`
// (upd < 0: initialise them with the payoff at the last date), then
// accumulate the regression of date `gram` (gram < 0: none).
template <class Real, int M, int B>
__device__ __forceinline__ void lsm_step_block(const LsmArgs &A, int upd, int gram, unsigned blk, unsigned nblk,
                                               double *red, bool &last) {
    constexpr int NA = M * (M + 1) / 2;
    constexpr int NS = NA + M + 1;  // A upper triangle, A^T y, ITM count
    const KxProgram &P = *A.P;
    const Real *S = reinterpret_cast<const Real *>(A.S);
    Real *V = reinterpret_cast<Real *>(A.value);
    constexpr bool F32 = sizeof(Real) == 4;
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
        have = A.coef[upd * LSM_COEF + 7] != 0.0;
#pragma unroll
        for (int j = 0; j < M; ++j) {
            cu[j] = A.coef[upd * LSM_COEF + j];
            cuf[j] = (float)cu[j];
        }
    }
    const float inv_scale = (float)(1.0 / A.x_scale);
    const LsmPay<Real> terms = lsm_pay_terms<Real>(P);
    const double disc_u = upd >= 0 ? A.disc[upd] : 0.0;
    const float disc_uf = (float)disc_u;
    const double disc_g = gram >= 0 ? A.disc[gram] : 0.0;
    const float disc_gf = (float)disc_g;
    for (uint64_t i = blk * (uint64_t)blockDim.x + threadIdx.x; i < A.n_paths; i += (uint64_t)nblk * blockDim.x) {
        Real val;
        if (upd < 0) {
            val = lsm_pay<Real>(terms, P, S[(uint64_t)(A.n_ex - 1) * A.n_paths + i], A.n_ex);
        } else if (F32) {  // the decision in FP32 (FP64 only across threads)
            const float s = (float)S[(uint64_t)upd * A.n_paths + i];
            const float pay = (float)lsm_pay<Real>(terms, P, (Real)s, upd + 1);
            const float discounted = (float)V[i] * disc_uf;
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
            const Real s = S[(uint64_t)upd * A.n_paths + i];
            const Real pay = lsm_pay<Real>(terms, P, s, upd + 1);
            const double discounted = (double)V[i] * disc_u;
            double nv = discounted;
            if (pay > Real(0)) {
                double cont = discounted;
                if (have) cont = lsm_continuation<M, B>(cu, (double)s, A.x_scale);
                nv = (double)pay > cont ? (double)pay : discounted;
            }
            val = (Real)nv;
        }
        V[i] = val;
        if (gram >= 0) {
            const Real sg = S[(uint64_t)gram * A.n_paths + i];
            if (lsm_pay<Real>(terms, P, sg, gram + 1) > Real(0)) {
                if (F32) {
                    const float yf = (float)val * disc_gf;
                    float pw[M];
                    lsm_basis_f32<M, B>((float)sg * inv_scale, pw);
                    int q = 0;
#pragma unroll
                    for (int r = 0; r < M; ++r)
#pragma unroll
                        for (int c = r; c < M; ++c) accf[q++] += pw[r] * pw[c];
#pragma unroll
                    for (int r = 0; r < M; ++r) accf[NA + r] += pw[r] * yf;
                    accf[NS - 1] += 1.0f;
                } else {
                    const double x = (double)sg;
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
    if (gram < 0) return;
    if (F32) block_sums_f32(accf, NS, red);
    else block_sums(acc, NS, red);
    if (threadIdx.x < NS) A.partial[(size_t)blk * 64 + threadIdx.x] = red[32 * 64 + threadIdx.x];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(A.ticket, 1u) == nblk - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // cross-block sums in a fixed order: 8 threads per sum, thread t of sum q
    // adds blocks t, t + 8, ... into 4 interleaved FP64 accumulators (the
    // FP64 pipe is slow; independent chains keep it busy), then the 4 and the
    // 8 partial sums are added in a fixed tree (deterministic)
    static_assert(NS * 8 <= LSM_BLOCK, "8 threads per sum");
    {
        const int q = threadIdx.x >> 3, t = threadIdx.x & 7;
        double s4[4] = {0.0, 0.0, 0.0, 0.0};
        if (q < NS) {
            unsigned b = t;
            for (; b + 24 < nblk; b += 32) {
#pragma unroll
                for (int u = 0; u < 4; ++u) s4[u] += __ldcg(A.partial + (size_t)(b + 8 * u) * 64 + q);
            }
            for (int u = 0; b < nblk; b += 8, u = (u + 1) & 3) s4[u] += __ldcg(A.partial + (size_t)b * 64 + q);
        }
        double v = (s4[0] + s4[1]) + (s4[2] + s4[3]);
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);  // within the 8 lanes of sum q
        if (q < NS && t == 0) red[q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // the solve on warp 0
        const double count = red[NS - 1];
        const bool fit = count >= (double)M;  // lsm.rs:190-194
        double x[LSM_MAXM];
        if (fit) solve_gauss_warp<M>(red, NA, x);
        if (threadIdx.x == 0) {
            for (int j = 0; j < M; ++j) A.coef[gram * LSM_COEF + j] = fit ? x[j] : 0.0;
            A.coef[gram * LSM_COEF + 7] = fit ? 1.0 : 0.0;
            *A.ticket = 0u;
        }
    }
}

template <class Real, int M, int B>
__global__ void __launch_bounds__(LSM_BLOCK, 4) k_lsm_step(const LsmArgs A, int upd, int gram) {
    __shared__ double red[32 * 64 + 64];
    __shared__ bool last;
    lsm_step_block<Real, M, B>(A, upd, gram, blockIdx.x, gridDim.x, red, last);
}

// One backward step of a batch of independent problems (cases): the cases
// still active at backward iteration `it` (case q of the launch owns blocks
// first[q] .. first[q + 1] - 1), each with its own dates, tables, partial
// sums, ticket and solve. A case's blocks compute exactly what the
// single-case launch of the same iteration computes.
template <class Real, int M, int B>
__global__ void __launch_bounds__(LSM_BLOCK, 4) k_lsm_step_batch(const LsmArgs *__restrict__ cases,
                                                                  const int *__restrict__ active,
                                                                  const unsigned *__restrict__ first, int n_active,
                                                                  int it) {
    __shared__ double red[32 * 64 + 64];
    __shared__ bool last;
    int lo = 0, hi = n_active - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const LsmArgs &A = cases[active[lo]];
    const int upd = it == 0 ? -1 : A.n_ex - 1 - it;
    const int gram = A.n_ex - 2 - it;
    lsm_step_block<Real, M, B>(A, upd, gram, blockIdx.x - first[lo], first[lo + 1] - first[lo], red, last);
}

template <class Real>
__global__ void __launch_bounds__(LSM_BLOCK) k_lsm_final(const LsmArgs A) {
    const Real *V = reinterpret_cast<const Real *>(A.value);
    const double d0 = A.disc[A.n_ex - 1];
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < A.n_paths;
         i += (uint64_t)gridDim.x * blockDim.x)
        A.pv[i] = (double)V[i] * d0;
}

template <class Real, int M, int B>
static void launch_steps_b(Ctx &c, const LsmArgs &a, int blocks) {
    const int n_ex = a.n_ex;
    k_lsm_step<Real, M, B><<<blocks, LSM_BLOCK, 0, c.stream>>>(a, -1, n_ex - 2);
    KX_CUDA(cudaGetLastError());
    c.last.kernel_launches++;
    for (int d = n_ex - 2; d >= 0; --d) {
        k_lsm_step<Real, M, B><<<blocks, LSM_BLOCK, 0, c.stream>>>(a, d, d - 1);
        KX_CUDA(cudaGetLastError());
        c.last.kernel_launches++;
    }
}

template <class Real, int M>
static void launch_steps(Ctx &c, const LsmArgs &a, int blocks, int basis) {
    if (basis == KX_LSM_LAGUERRE) launch_steps_b<Real, M, KX_LSM_LAGUERRE>(c, a, blocks);
    else launch_steps_b<Real, M, KX_LSM_MONOMIAL>(c, a, blocks);
}

template <class Real>
static void run_lsm(Ctx &c, LsmArgs &a, int m, int model, int basis) {
    const int blocks = c.sm_count * 4;
    if (model == KX_MODEL_GBM) k_lsm_forward<Real, KX_MODEL_GBM><<<blocks, LSM_BLOCK, 0, c.stream>>>(a);
    else k_lsm_forward<Real, KX_MODEL_HESTON><<<blocks, LSM_BLOCK, 0, c.stream>>>(a);
    KX_CUDA(cudaGetLastError());
    c.last.kernel_launches++;
    switch (m) {
    case 2: launch_steps<Real, 2>(c, a, blocks, basis); break;
    case 3: launch_steps<Real, 3>(c, a, blocks, basis); break;
    case 4: launch_steps<Real, 4>(c, a, blocks, basis); break;
    case 5: launch_steps<Real, 5>(c, a, blocks, basis); break;
    default: launch_steps<Real, 6>(c, a, blocks, basis); break;
    }
    k_lsm_final<Real><<<blocks, LSM_BLOCK, 0, c.stream>>>(a);
    KX_CUDA(cudaGetLastError());
    c.last.kernel_launches++;
}

// Host tables of one LSM problem (validation as lsm.rs:87-105).
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
    return L;
}

template <class Real, int M, int B>
static void launch_batch_b(Ctx &c, const LsmArgs *cases, const std::vector<int> &n_ex, int blocks, void *idx_dev) {
    const int n = (int)n_ex.size();
    const int max_ex = *std::max_element(n_ex.begin(), n_ex.end());
    const int *act = static_cast<const int *>(idx_dev);
    // the active cases of every iteration, uploaded once: row `it` = [case ids..., block starts...]
    std::vector<int> rows((size_t)max_ex * (2 * n + 1), 0);
    std::vector<int> counts(max_ex, 0);
    for (int it = 0; it < max_ex; ++it) {
        int *row = rows.data() + (size_t)it * (2 * n + 1);
        int q = 0;
        for (int i = 0; i < n; ++i)
            if (it <= n_ex[i] - 1) row[q++] = i;
        for (int j = 0; j <= q; ++j) row[n + j] = j * blocks;
        counts[it] = q;
    }
    KX_CUDA(cudaMemcpyAsync(idx_dev, rows.data(), rows.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    for (int it = 0; it < max_ex; ++it) {
        const int *row = act + (size_t)it * (2 * n + 1);
        const unsigned *fst = reinterpret_cast<const unsigned *>(row + n);
        k_lsm_step_batch<Real, M, B><<<counts[it] * blocks, LSM_BLOCK, 0, c.stream>>>(cases, row, fst, counts[it], it);
        KX_CUDA(cudaGetLastError());
        c.last.kernel_launches++;
    }
}

template <class Real, int M>
static void launch_batch(Ctx &c, const LsmArgs *cases, const std::vector<int> &n_ex, int blocks, void *idx, int basis) {
    if (basis == KX_LSM_LAGUERRE) launch_batch_b<Real, M, KX_LSM_LAGUERRE>(c, cases, n_ex, blocks, idx);
    else launch_batch_b<Real, M, KX_LSM_MONOMIAL>(c, cases, n_ex, blocks, idx);
}

template <class Real>
static void run_lsm_batch(Ctx &c, std::vector<LsmCase> &cs, const LsmArgs *cases_dev, int m, int basis,
                          void *idx_dev) {
    const int blocks = c.sm_count * 4;
    for (auto &L : cs) {  // forward simulations (each writes its own S)
        if (L.np == 0) continue;
        if (L.m.kind == KX_MODEL_GBM) k_lsm_forward<Real, KX_MODEL_GBM><<<blocks, LSM_BLOCK, 0, c.stream>>>(L.a);
        else k_lsm_forward<Real, KX_MODEL_HESTON><<<blocks, LSM_BLOCK, 0, c.stream>>>(L.a);
        KX_CUDA(cudaGetLastError());
        c.last.kernel_launches++;
    }
    std::vector<int> n_ex;
    for (auto &L : cs) n_ex.push_back(L.np ? L.n_ex : 0);  // a case without paths is never active
    switch (m) {
    case 2: launch_batch<Real, 2>(c, cases_dev, n_ex, blocks, idx_dev, basis); break;
    case 3: launch_batch<Real, 3>(c, cases_dev, n_ex, blocks, idx_dev, basis); break;
    case 4: launch_batch<Real, 4>(c, cases_dev, n_ex, blocks, idx_dev, basis); break;
    case 5: launch_batch<Real, 5>(c, cases_dev, n_ex, blocks, idx_dev, basis); break;
    default: launch_batch<Real, 6>(c, cases_dev, n_ex, blocks, idx_dev, basis); break;
    }
    for (auto &L : cs) {
        if (L.np == 0) continue;
        k_lsm_final<Real><<<blocks, LSM_BLOCK, 0, c.stream>>>(L.a);
        KX_CUDA(cudaGetLastError());
        c.last.kernel_launches++;
    }
}

}  // namespace kx

using namespace kx;

extern "C" kx_status kx_price_american_lsm_basis(const kx_program *prog, const kx_model *model,
                                                 const kx_mc_config *cfg, const double *dates, size_t n_dates,
                                                 int32_t n_basis, int32_t basis, kx_price_result *out) {
    return guarded([&] {
        if (!out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        LsmCase L = lsm_case(prog, model, cfg, dates, n_dates, n_basis, basis);
        const bool f64 = cfg->precision == KX_PREC_FP64;
        const uint64_t np = L.np;
        const int n_ex = L.n_ex;
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        const size_t rs = f64 ? 8 : 4;
        const int blocks = c.sm_count * 4;
        c.progs.ensure(sizeof(KxProgram));
        c.steps.ensure(L.steps.size());
        c.disc.ensure(L.disc.size() * sizeof(double));
        c.lsm_paths.ensure(std::max<uint64_t>(1, np * n_ex) * rs);
        c.lsm_value.ensure(std::max<uint64_t>(1, np) * rs);
        c.pv.ensure(std::max<uint64_t>(1, np) * sizeof(double));
        c.lsm_stats.ensure((size_t)blocks * 64 * sizeof(double) + (size_t)n_ex * LSM_COEF * sizeof(double));
        c.counters.ensure(64);
        KX_CUDA(cudaMemcpyAsync(c.progs.p, &L.P, sizeof L.P, cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync(c.steps.p, L.steps.data(), L.steps.size(), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync(c.disc.p, L.disc.data(), L.disc.size() * sizeof(double), cudaMemcpyHostToDevice,
                                c.stream));
        KX_CUDA(cudaMemsetAsync(c.counters.p, 0, 64, c.stream));
        c.last.h2d_bytes += sizeof L.P + L.steps.size() + L.disc.size() * sizeof(double);
        LsmArgs &a = L.a;
        a.P = c.progs.as<KxProgram>();
        a.steps = c.steps.p;
        a.disc = c.disc.as<double>();
        if (cfg->rng == KX_RNG_SHARED_DRAWS) {
            DrawStore &ds = c.draws;
            if (!ds.set) raise(KX_INVALID_ARGUMENT, "no shared draws registered");
            if (ds.n_paths < np || ds.dpp < (uint64_t)n_ex * L.m.draws_per_step())
                raise(KX_INVALID_ARGUMENT, "shared draws too small for this simulation");
            a.z64 = ds.is64 ? ds.z64.as<double>() : nullptr;
            a.z32 = ds.is64 ? nullptr : ds.z32.as<float>();
            a.z_dpp = ds.dpp;
        }
        a.S = c.lsm_paths.p;
        a.value = c.lsm_value.p;
        a.pv = c.pv.as<double>();
        a.partial = c.lsm_stats.as<double>();
        a.coef = c.lsm_stats.as<double>() + (size_t)blocks * 64;
        a.ticket = c.counters.as<unsigned>();
        if (np > 0) {
            KX_CUDA(cudaEventRecord(c.ev0, c.stream));
            if (f64) run_lsm<double>(c, a, n_basis, L.m.kind, basis);
            else run_lsm<float>(c, a, n_basis, L.m.kind, basis);
            KX_CUDA(cudaEventRecord(c.ev1, c.stream));
            KX_CUDA(cudaEventSynchronize(c.ev1));
            float ms = 0.f;
            KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
            c.last.kernel_ms += ms;
        }
        c.last.path_steps += np * (uint64_t)n_ex;
        c.last.steps_simulated += np * (uint64_t)n_ex;
        std::vector<StatsJob> sj(1);
        sj[0].n = np;
        *out = finish(device_stats(c, c.pv.as<double>(), np, sj)[0]);
        c.last.total_ms += now_ms();
    });
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
        std::vector<LsmCase> cs;
        for (size_t i = 0; i < n; ++i) {
            cs.push_back(lsm_case(progs[i], &models[i], &cfgs[i], dates[i], n_dates[i], n_basis, basis));
            if (cfgs[i].rng != KX_RNG_PHILOX) raise(KX_INVALID_ARGUMENT, "an LSM batch draws from Philox");
            if (cfgs[i].precision != cfgs[0].precision) raise(KX_INVALID_ARGUMENT, "an LSM batch has one precision");
        }
        const bool f64 = cfgs[0].precision == KX_PREC_FP64;
        const size_t rs = f64 ? 8 : 4;
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        const int blocks = c.sm_count * 4;
        // one arena: per case its program, steps, discounts, paths, values, per-path results,
        // partial sums, coefficients and ticket; then the case table and the iteration table
        auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
        std::vector<size_t> off(n + 1, 0);
        uint64_t tot_paths = 0;
        int max_ex = 0;
        for (size_t i = 0; i < n; ++i) {
            const LsmCase &L = cs[i];
            size_t b = al(sizeof(KxProgram)) + al(L.steps.size()) + al(L.disc.size() * sizeof(double)) +
                       al(std::max<uint64_t>(1, L.np * L.n_ex) * rs) + al(std::max<uint64_t>(1, L.np) * rs) +
                       al(std::max<uint64_t>(1, L.np) * sizeof(double)) + al((size_t)blocks * 64 * sizeof(double)) +
                       al((size_t)L.n_ex * LSM_COEF * sizeof(double)) + al(64);
            off[i + 1] = off[i] + b;
            tot_paths += L.np;
            max_ex = std::max(max_ex, L.n_ex);
        }
        const size_t off_cases = off[n], off_idx = al(off_cases + n * sizeof(LsmArgs));
        const size_t total = al(off_idx + (size_t)max_ex * (2 * n + 1) * sizeof(int));
        c.lsm_paths.ensure(total);
        unsigned char *base = c.lsm_paths.as<unsigned char>();
        std::vector<LsmArgs> args(n);
        std::vector<StatsJob> sj(n);
        for (size_t i = 0; i < n; ++i) {
            LsmCase &L = cs[i];
            unsigned char *q = base + off[i];
            auto take = [&](size_t bytes) { unsigned char *r = q; q += al(bytes); return r; };
            L.a.P = reinterpret_cast<const KxProgram *>(take(sizeof(KxProgram)));
            L.a.steps = take(L.steps.size());
            L.a.disc = reinterpret_cast<const double *>(take(L.disc.size() * sizeof(double)));
            L.a.S = take(std::max<uint64_t>(1, L.np * L.n_ex) * rs);
            L.a.value = take(std::max<uint64_t>(1, L.np) * rs);
            L.a.pv = reinterpret_cast<double *>(take(std::max<uint64_t>(1, L.np) * sizeof(double)));
            L.a.partial = reinterpret_cast<double *>(take((size_t)blocks * 64 * sizeof(double)));
            L.a.coef = reinterpret_cast<double *>(take((size_t)L.n_ex * LSM_COEF * sizeof(double)));
            L.a.ticket = reinterpret_cast<unsigned *>(take(64));
            KX_CUDA(cudaMemcpyAsync((void *)L.a.P, &L.P, sizeof(KxProgram), cudaMemcpyHostToDevice, c.stream));
            KX_CUDA(cudaMemcpyAsync((void *)L.a.steps, L.steps.data(), L.steps.size(), cudaMemcpyHostToDevice, c.stream));
            KX_CUDA(cudaMemcpyAsync((void *)L.a.disc, L.disc.data(), L.disc.size() * sizeof(double),
                                    cudaMemcpyHostToDevice, c.stream));
            KX_CUDA(cudaMemsetAsync(L.a.ticket, 0, 64, c.stream));
            c.last.h2d_bytes += sizeof(KxProgram) + L.steps.size() + L.disc.size() * sizeof(double);
            args[i] = L.a;
            sj[i].begin = (uint64_t)(reinterpret_cast<unsigned char *>(L.a.pv) - base) / sizeof(double);
            sj[i].n = L.np;
            c.last.path_steps += L.np * (uint64_t)L.n_ex;
        }
        LsmArgs *cases_dev = reinterpret_cast<LsmArgs *>(base + off_cases);
        KX_CUDA(cudaMemcpyAsync(cases_dev, args.data(), n * sizeof(LsmArgs), cudaMemcpyHostToDevice, c.stream));
        c.last.steps_simulated = c.last.path_steps;
        if (tot_paths > 0) {
            KX_CUDA(cudaEventRecord(c.ev0, c.stream));
            if (f64) run_lsm_batch<double>(c, cs, cases_dev, n_basis, basis, base + off_idx);
            else run_lsm_batch<float>(c, cs, cases_dev, n_basis, basis, base + off_idx);
            KX_CUDA(cudaEventRecord(c.ev1, c.stream));
            KX_CUDA(cudaEventSynchronize(c.ev1));
            float ms = 0.f;
            KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
            c.last.kernel_ms += ms;
        }
        auto st = device_stats(c, reinterpret_cast<const double *>(base), 0, sj);
        for (size_t i = 0; i < n; ++i) out[i] = finish(st[i]);
        c.last.total_ms += now_ms();
    });
}
