// device_common.cuh — device building blocks shared by the path kernels:
// counter-based normals, the postfix expression interpreter and the
// accumulator (Average / RunningMax / RunningMin) semantics.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/kontract_gpu.h"
#include "devprog.hpp"

namespace kx {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011): 10 rounds of two 32x32->64 multiplies with a
// Weyl-sequence key schedule. Counter = (block, path_lo, path_hi, stream),
// key = (seed_lo, seed_hi).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x;
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Philox4x32-10 with its round keys given: rk[2r] = k0 + r * 0x9E3779B9,
// rk[2r + 1] = k1 + r * 0xBB67AE85 (the key schedule above, precomputed on
// the host). Kept in kernel parameters, the keys are constant-bank operands
// of the XORs, so the 20 key additions of a call disappear.
__device__ __forceinline__ uint4 philox4x32_10_rk(uint4 c, const uint32_t (&rk)[20]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x;
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ rk[2 * r], lo1, hi0 ^ c.w ^ rk[2 * r + 1], lo0);
    }
    return c;
}

// The round keys of one seed for philox4x32_10_rk, passed to a kernel as a
// parameter when every path of the launch draws from that seed (ok = 1).
struct PhiloxKeys {
    uint32_t ok;
    uint32_t rk[20];
};

inline PhiloxKeys philox_keys(uint64_t seed) {
    PhiloxKeys K{};
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        K.rk[2 * r] = k0;
        K.rk[2 * r + 1] = k1;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    K.ok = 1u;
    return K;
}

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Box-Muller on two 32-bit words: u = (w + 1/2) 2^-32 in (0, 1),
// z0 = r cos(2 pi u2), z1 = r sin(2 pi u2), r = sqrt(-2 ln u1).
// FP32: the angle is taken as 2 pi (u2 - 1/2) in (-pi, pi), the range where
// the hardware sine/cosine are accurate, and the sign is folded back.
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float &z0, float &z1) {
    const float u1 = fmaf(__uint2float_rn(a), 0x1p-32f, 0x1p-33f);
    const float h = fmaf(__uint2float_rn(b), 0x1p-32f, 0x1p-33f - 0.5f);
    const float r = sqrt_approx(-2.0f * __logf(u1));
    float s, c;
    __sincosf(6.283185307179586f * h, &s, &c);
    z0 = -r * c;
    z1 = -r * s;
}
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, double &z0, double &z1) {
    const double u1 = ((double)a + 0.5) * 0x1p-32;
    const double u2 = ((double)b + 0.5) * 0x1p-32;
    const double r = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

template <class Real>
__device__ __forceinline__ Real fast_exp(Real x);
template <>
__device__ __forceinline__ float fast_exp<float>(float x) { return __expf(x); }
template <>
__device__ __forceinline__ double fast_exp<double>(double x) { return exp(x); }

// Next representable value up / down (a strict comparison with t is the
// inclusive one with the neighbour of t).
__device__ __forceinline__ float next_up(float t) { return nextafterf(t, INFINITY); }
__device__ __forceinline__ double next_up(double t) { return ::nextafter(t, (double)INFINITY); }
__device__ __forceinline__ float next_down(float t) { return nextafterf(t, -INFINITY); }
__device__ __forceinline__ double next_down(double t) { return ::nextafter(t, -(double)INFINITY); }

// The logistic 1 / (1 + e^x) of a smoothed barrier (FP32: hardware exp and
// the approximate divide; every kernel that weighs a path uses this one).
__device__ __forceinline__ float logistic(float x) { return __fdividef(1.0f, 1.0f + __expf(x)); }
__device__ __forceinline__ double logistic(double x) { return 1.0 / (1.0 + exp(x)); }

// The weight of one step under a smoothed barrier, logistic(x) with x the
// signed distance past the barrier in widths. Where 1 + e^x rounds to 1 in
// the arithmetic's precision (e^x below half an ulp of 1: x <= -17 in FP32,
// x <= -38 in FP64) the weight is exactly 1, so a kernel may skip those steps
// and still agree bit for bit with one that evaluates them.
template <class Real> __device__ __forceinline__ Real smooth_cut();
template <> __device__ __forceinline__ float smooth_cut<float>() { return -17.0f; }
template <> __device__ __forceinline__ double smooth_cut<double>() { return -38.0; }
template <class Real>
__device__ __forceinline__ Real smooth_weight(Real x) {
    return x <= smooth_cut<Real>() ? Real(1) : logistic(x);
}

// Separately rounded arithmetic in either precision (never fused into an FMA).
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Amount of a flow slot with a closed form (KxFastAmount): the operations of
// the interpreter on its code, in the same order, so the value is identical.
template <class Real>
__device__ __forceinline__ Real fast_amount(const KxProgram &P, const KxLeaf &F, Real S) {
    const Real K = (Real)P.cpool[F.fast_k];
    Real r;
    switch (F.fast) {
    case FA_CALL: r = fmax(S - K, Real(0)); break;
    case FA_PUT: r = fmax(K - S, Real(0)); break;
    case FA_SPOT: r = S; break;
    default: r = K; break;
    }
    return F.sign < 0.0 ? -r : r;
}

// One log-space GBM step y += c0 + c1 z with its roundings fixed (one FMA,
// one add), identical in every kernel that steps a path.
__device__ __forceinline__ float gbm_step(float y, float c0, float c1, float z) {
    return __fadd_rn(y, __fmaf_rn(c1, z, c0));
}
__device__ __forceinline__ double gbm_step(double y, double c0, double c1, double z) {
    return __dadd_rn(y, __fma_rn(c1, z, c0));
}

// S = s0 * exp(y) rounded once, so that no later use is fused into an FMA
// with it: every kernel then sees the same S bit for bit.
template <class Real>
__device__ __forceinline__ Real spot_of(Real s0, Real y);
template <>
__device__ __forceinline__ float spot_of<float>(float s0, float y) { return __fmul_rn(s0, __expf(y)); }
template <>
__device__ __forceinline__ double spot_of<double>(double s0, double y) { return __dmul_rn(s0, exp(y)); }

// ---------------------------------------------------------------------------
// Accumulators live in shared memory, one column per thread:
// slot j of this thread is base[j * stride].
// ---------------------------------------------------------------------------
template <class Real>
struct AccView {
    Real *base;
    int stride;
    __device__ __forceinline__ Real &operator[](int j) const { return base[j * stride]; }
};

// Value of accumulator `a` read at step k (observable.rs:103-140).
// err gets KX_ERR_* bits when the reference would fail there.
template <class Real>
__device__ __forceinline__ Real acc_value(const KxProgram &P, int a, AccView<Real> acc, uint32_t poisoned, int k,
                                          uint32_t &err) {
    const KxAcc &A = P.acc[a];
    if (poisoned >> a & 1u) err |= KX_ERR_MALFORMED;
    const Real v = acc[a];
    if (A.kind != ACC_SUM) return v;
    if (A.fixed) {
        if (A.static_err) { err |= KX_ERR_MALFORMED; return Real(0); }
        if (k < A.e_min) { err |= KX_ERR_LOOKAHEAD; return Real(0); }
        return v / (Real)A.inv_count;
    }
    if (k < A.e_min) { err |= KX_ERR_MALFORMED; return Real(0); }
    return v / (Real)(k - A.i_from + 1);
}

// Postfix interpreter. Reals and booleans share one stack (booleans as 0/1);
// `em` keeps one error bit per stack slot so that errors propagate the way
// the reference's `?` operators do, including the short-circuit of
// `a && b` / `a || b` (observable.rs:164-165).
template <class Real>
struct EvalOut {
    Real v;
    uint32_t err;
};

template <class Real>
__device__ __noinline__ EvalOut<Real> eval_code_impl(const KxProgram *__restrict__ Pp, int off, int len, Real *acc_base,
                                                     int acc_stride, uint32_t poisoned, int k, Real S,
                                                     const Real *Sx) {
    const KxProgram &P = *Pp;
    const AccView<Real> acc{acc_base, acc_stride};
    Real st[KX_MAX_STACK];
    uint32_t eb[KX_MAX_STACK];
    int sp = 0;
    for (int pc = off; pc < off + len; ++pc) {
        const KxIns ins = P.code[pc];
        switch (ins.op) {
        case OP_CONST: st[sp] = (Real)P.cpool[ins.arg]; eb[sp++] = 0; break;
        case OP_SPOT: st[sp] = Sx ? Sx[ins.arg] : S; eb[sp++] = 0; break;  // Sx: the spots of a multi-asset path
        case OP_ACC: {
            uint32_t e = 0;
            st[sp] = acc_value<Real>(P, ins.arg, acc, poisoned, k, e);
            eb[sp++] = e;
            break;
        }
        case OP_NEG: st[sp - 1] = -st[sp - 1]; break;
        case OP_TRUE: st[sp] = Real(1); eb[sp++] = 0; break;
        case OP_FALSE: st[sp] = Real(0); eb[sp++] = 0; break;
        case OP_AT: st[sp] = k >= P.at_index[ins.arg] ? Real(1) : Real(0); eb[sp++] = 0; break;
        case OP_NOT: st[sp - 1] = st[sp - 1] != Real(0) ? Real(0) : Real(1); break;
        default: {
            --sp;
            const Real a = st[sp - 1], b = st[sp];
            const uint32_t ea = eb[sp - 1], ebb = eb[sp];
            Real r;
            uint32_t e = ea | ebb;
            switch (ins.op) {
            case OP_ADD: r = a + b; break;
            case OP_SUB: r = a - b; break;
            case OP_MUL: r = a * b; break;
            case OP_DIV: r = a / b; break;
            case OP_MAX: r = fmax(a, b); break;
            case OP_MIN: r = fmin(a, b); break;
            case OP_GE: r = a >= b ? Real(1) : Real(0); break;
            case OP_GT: r = a > b ? Real(1) : Real(0); break;
            case OP_LE: r = a <= b ? Real(1) : Real(0); break;
            case OP_LT: r = a < b ? Real(1) : Real(0); break;
            case OP_AND: r = (a != Real(0) && b != Real(0)) ? Real(1) : Real(0); e = ea | (a != Real(0) ? ebb : 0u); break;
            case OP_OR: r = (a != Real(0) || b != Real(0)) ? Real(1) : Real(0); e = ea | (a == Real(0) ? ebb : 0u); break;
            default: r = Real(0); break;
            }
            st[sp - 1] = r;
            eb[sp - 1] = e;
            break;
        }
        }
    }
    return EvalOut<Real>{st[0], eb[0]};
}

// Out-of-line so the (rare) interpreter does not weigh on the registers of
// the per-step path that calls it.
template <class Real>
__device__ __forceinline__ Real eval_code(const KxProgram &P, int off, int len, AccView<Real> acc, uint32_t poisoned,
                                          int k, Real S, uint32_t &err, const Real *Sx = nullptr) {
    const EvalOut<Real> o = eval_code_impl<Real>(&P, off, len, acc.base, acc.stride, poisoned, k, S, Sx);
    err |= o.err;
    return o.v;
}

template <class Real>
struct StepRec {  // grid step k (k = 0 carries only the time bits)
    Real c0, c1;  // GBM single scenario: drift*dt, sigma*sqrt(dt); otherwise dt, sqrt(dt)
    uint32_t tt;  // CK_TIME trigger bits true at step k
    uint32_t pad;
};

template <class Real> __device__ __forceinline__ Real pick(double d, float f);
template <> __device__ __forceinline__ float pick<float>(double, float f) { return f; }
template <> __device__ __forceinline__ double pick<double>(double d, float) { return d; }

template <class Real> __device__ __forceinline__ Real fsqrt(Real x);
template <> __device__ __forceinline__ float fsqrt<float>(float x) { return sqrt_approx(x); }
template <> __device__ __forceinline__ double fsqrt<double>(double x) { return sqrt(x); }

// Heston Euler step (simulator.rs:506-541) in log-spot; dt and sqrt(dt) come
// from the step table. The variance update keeps the reference's operation
// order without fused multiply-adds in FP64, so on shared normals it rounds
// exactly like the reference (v near 0 feeds sqrt, which would magnify any
// rounding difference). REFERENCE_FLOOR floors v after the step; full
// truncation (Lord et al. 2010) uses max(v, 0) inside the step instead.
template <class Real>
__device__ __forceinline__ void heston_step(Real r, Real kap, Real th, Real sv, Real rho, Real rp, int scheme, Real dt,
                                            Real sq, Real z1, Real z2, Real &y, Real &v);
template <>
__device__ __forceinline__ void heston_step<float>(float r, float kap, float th, float sv, float rho, float rp,
                                                   int scheme, float dt, float sq, float z1, float z2, float &y,
                                                   float &v) {
    // every rounding spelled out, so that no kernel fuses it differently
    const float vp = scheme == KX_HESTON_FULL_TRUNCATION ? fmaxf(v, 0.f) : v;
    const float sqv = sqrt_approx(vp);
    const float drift = __fmaf_rn(__fmul_rn(-0.5f, vp), dt, __fmul_rn(r, dt));  // (r - v/2) dt
    y = __fadd_rn(y, __fmaf_rn(sqv, __fmul_rn(z1, sq), drift));
    const float zv = __fmaf_rn(rho, z1, __fmul_rn(rp, z2));
    const float nv = __fmaf_rn(__fmul_rn(sv, sqv), __fmul_rn(zv, sq), __fmaf_rn(__fmul_rn(kap, __fsub_rn(th, vp)), dt, v));
    v = scheme == KX_HESTON_FULL_TRUNCATION ? nv : fmaxf(nv, 0.f);
}
template <>
__device__ __forceinline__ void heston_step<double>(double r, double kap, double th, double sv, double rho, double rp,
                                                    int scheme, double dt, double sq, double z1, double z2, double &y,
                                                    double &v) {
    const double vp = scheme == KX_HESTON_FULL_TRUNCATION ? fmax(v, 0.0) : v;
    const double sqv = sqrt(vp);
    const double dw_s = __dmul_rn(z1, sq);
    const double dw_v = __dmul_rn(__dadd_rn(__dmul_rn(rho, z1), __dmul_rn(rp, z2)), sq);
    y += __dadd_rn(__dsub_rn(__dmul_rn(r, dt), __dmul_rn(__dmul_rn(0.5, vp), dt)), __dmul_rn(sqv, dw_s));
    const double nv = __dadd_rn(__dadd_rn(v, __dmul_rn(__dmul_rn(kap, __dsub_rn(th, vp)), dt)),
                                __dmul_rn(__dmul_rn(sv, sqv), dw_v));
    v = scheme == KX_HESTON_FULL_TRUNCATION ? nv : (nv != nv ? 0.0 : fmax(nv, 0.0));
}

}  // namespace kx
