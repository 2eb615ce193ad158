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

// numerics.rs:190-236 for m <= LSM_MAXM, on one thread.
__device__ void solve_gauss(double a[LSM_MAXM][LSM_MAXM], double b[LSM_MAXM], int m, double x[LSM_MAXM]) {
    for (int col = 0; col < m; ++col) {
        int piv = col;
        double best = fabs(a[col][col]);
        for (int row = col + 1; row < m; ++row) {
            const double v = fabs(a[row][col]);
            if (v > best) { best = v; piv = row; }
        }
        if (best < 1e-12) {
            for (int j = 0; j < m; ++j) x[j] = 0.0;
            return;
        }
        for (int c = 0; c < m; ++c) { const double t = a[col][c]; a[col][c] = a[piv][c]; a[piv][c] = t; }
        { const double t = b[col]; b[col] = b[piv]; b[piv] = t; }
        for (int row = col + 1; row < m; ++row) {
            const double factor = __ddiv_rn(a[row][col], a[col][col]);
            for (int c = col; c < m; ++c) a[row][c] = __dsub_rn(a[row][c], __dmul_rn(factor, a[col][c]));
            b[row] = __dsub_rn(b[row], __dmul_rn(factor, b[col]));
        }
    }
    for (int row = m - 1; row >= 0; --row) {
        double sum = b[row];
        for (int c = row + 1; c < m; ++c) sum = __dsub_rn(sum, __dmul_rn(a[row][c], x[c]));
        x[row] = __ddiv_rn(sum, a[row][row]);
    }
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

// One backward launch: update the values with the decision of date `upd`
// (upd < 0: initialise them with the payoff at the last date), then
// accumulate the regression of date `gram` (gram < 0: none).
template <class Real, int M, int B>
__global__ void __launch_bounds__(LSM_BLOCK, 4) k_lsm_step(const LsmArgs A, int upd, int gram) {
    constexpr int NA = M * (M + 1) / 2;
    constexpr int NS = NA + M + 1;  // A upper triangle, A^T y, ITM count
    __shared__ double red[32 * 64 + 64];
    __shared__ bool last;
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
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < A.n_paths;
         i += (uint64_t)gridDim.x * blockDim.x) {
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
    if (threadIdx.x < NS) A.partial[(size_t)blockIdx.x * 64 + threadIdx.x] = red[32 * 64 + threadIdx.x];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(A.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // cross-block sums by the whole block: thread t adds blocks t, t + 256,
    // ... in that order, then the fixed-order block sum (deterministic)
    {
        double part[NS];
#pragma unroll
        for (int q = 0; q < NS; ++q) part[q] = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
            for (int q = 0; q < NS; ++q) part[q] += __ldcg(A.partial + (size_t)b * 64 + q);
        }
        block_sums(part, NS, red);
        if (threadIdx.x < NS) red[threadIdx.x] = red[32 * 64 + threadIdx.x];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a[LSM_MAXM][LSM_MAXM], b[LSM_MAXM], x[LSM_MAXM];
        int q = 0;
        for (int r = 0; r < M; ++r)
            for (int c = r; c < M; ++c) { a[r][c] = red[q]; a[c][r] = red[q]; ++q; }
        for (int r = 0; r < M; ++r) b[r] = red[NA + r];
        const double count = red[NS - 1];
        const bool fit = count >= (double)M;  // lsm.rs:190-194
        if (fit) solve_gauss(a, b, M, x);
        for (int j = 0; j < M; ++j) A.coef[gram * LSM_COEF + j] = fit ? x[j] : 0.0;
        A.coef[gram * LSM_COEF + 7] = fit ? 1.0 : 0.0;
        *A.ticket = 0u;
    }
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

}  // namespace kx

using namespace kx;

extern "C" kx_status kx_price_american_lsm_basis(const kx_program *prog, const kx_model *model,
                                                 const kx_mc_config *cfg, const double *dates, size_t n_dates,
                                                 int32_t n_basis, int32_t basis, kx_price_result *out) {
    return guarded([&] {
        if (basis != KX_LSM_MONOMIAL && basis != KX_LSM_LAGUERRE) raise(KX_INVALID_ARGUMENT, "unknown LSM basis");
        const Program &p = program_of(prog);
        Model m = model_from_c(model);
        if (!cfg || !out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        if (cfg->flags != 0 || (cfg->rng != KX_RNG_PHILOX && cfg->rng != KX_RNG_SHARED_DRAWS) ||
            (cfg->precision != KX_PREC_FP32 && cfg->precision != KX_PREC_FP64))
            raise(KX_INVALID_ARGUMENT, "bad config");
        // lsm.rs:87-105
        if (n_dates == 0 || !dates) raise(KX_MALFORMED_CONTRACT, "LSM: at least one exercise date required");
        for (size_t i = 1; i < n_dates; ++i)
            if (!(dates[i] > dates[i - 1])) raise(KX_MALFORMED_CONTRACT, "LSM: exercise dates must increase and be > 0");
        if (!(dates[0] > 0.0)) raise(KX_MALFORMED_CONTRACT, "LSM: exercise dates must increase and be > 0");
        if (n_basis < 2) raise(KX_MALFORMED_CONTRACT, "LSM: n_basis >= 2 required");
        if (n_basis > LSM_MAXM) raise(KX_UNSUPPORTED, "LSM: n_basis above 6 is not supported on the device");
        const KxProgram &L = p.low.prog;
        if (L.n_trig != 0 || L.n_acc != 0)
            raise(KX_UNSUPPORTED, "LSM payoff must be an immediate function of the spot "
                                  "(no when/until/anytime, averages or running extrema)");
        validate_model(m);
        std::vector<double> grid{0.0};
        grid.insert(grid.end(), dates, dates + n_dates);
        validate_grid(grid);
        const bool f64 = cfg->precision == KX_PREC_FP64;
        const uint64_t np = cfg->n_paths;
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        memset(&c.last, 0, sizeof c.last);
        c.last.total_ms = -now_ms();
        KxProgram P;
        StepTables tab;
        bind(p.low, grid, m, cfg->rate, P, tab);
        const int n_ex = (int)n_dates;
        std::vector<double> disc(n_ex);
        for (int d = 0; d + 1 < n_ex; ++d) disc[d] = std::exp(-cfg->rate * (dates[d + 1] - dates[d]));  // lsm.rs:176
        disc[n_ex - 1] = std::exp(-cfg->rate * dates[0]);                                            // lsm.rs:226
        std::vector<unsigned char> steps(grid.size() * (f64 ? sizeof(StepRec<double>) : sizeof(StepRec<float>)));
        for (size_t k = 0; k < grid.size(); ++k) {
            if (f64) reinterpret_cast<StepRec<double> *>(steps.data())[k] = {tab.c0[k], tab.c1[k], 0u, 0u};
            else reinterpret_cast<StepRec<float> *>(steps.data())[k] = {(float)tab.c0[k], (float)tab.c1[k], 0u, 0u};
        }
        const size_t rs = f64 ? 8 : 4;
        const int blocks = c.sm_count * 4;
        c.progs.ensure(sizeof(KxProgram));
        c.steps.ensure(steps.size());
        c.disc.ensure(disc.size() * sizeof(double));
        c.lsm_paths.ensure(std::max<uint64_t>(1, np * n_ex) * rs);
        c.lsm_value.ensure(std::max<uint64_t>(1, np) * rs);
        c.pv.ensure(std::max<uint64_t>(1, np) * sizeof(double));
        c.lsm_stats.ensure((size_t)blocks * 64 * sizeof(double) + (size_t)n_ex * LSM_COEF * sizeof(double));
        c.counters.ensure(64);
        KX_CUDA(cudaMemcpyAsync(c.progs.p, &P, sizeof P, cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync(c.steps.p, steps.data(), steps.size(), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync(c.disc.p, disc.data(), disc.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemsetAsync(c.counters.p, 0, 64, c.stream));
        c.last.h2d_bytes += sizeof P + steps.size() + disc.size() * sizeof(double);
        LsmArgs a{};
        a.P = c.progs.as<KxProgram>();
        a.steps = c.steps.p;
        a.disc = c.disc.as<double>();
        a.n_times = (int)grid.size();
        a.n_ex = n_ex;
        a.n_paths = np;
        a.seed = cfg->seed;
        a.model = m.kind;
        a.scheme = m.scheme;
        a.s0 = m.s0;
        a.v0 = m.v0; a.kappa = m.kappa; a.theta = m.theta; a.sigma_v = m.sigma_v; a.rho = m.rho;
        a.rho_perp = std::sqrt(std::max(1.0 - m.rho * m.rho, 0.0));
        a.r = m.r;
        a.x_scale = m.s0;
        if (cfg->rng == KX_RNG_SHARED_DRAWS) {
            DrawStore &ds = c.draws;
            if (!ds.set) raise(KX_INVALID_ARGUMENT, "no shared draws registered");
            if (ds.n_paths < np || ds.dpp < (uint64_t)n_ex * m.draws_per_step())
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
            if (f64) run_lsm<double>(c, a, n_basis, m.kind, basis);
            else run_lsm<float>(c, a, n_basis, m.kind, basis);
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
