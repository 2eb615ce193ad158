// engine.cu — the fused path kernel and the GPU entry points of the C ABI.
//
// One kernel (k_paths) replaces Gbm::simulate / HestonSimulator::simulate
// (src/simulator.rs:215-253, 506-541) + price_on_paths / cashflows
// (src/pricer.rs:230-433): each thread draws its normals from Philox in
// registers, advances the path state (log-spot, variance) one grid step at a
// time and interprets the lowered contract table at every step, so the path is
// never stored. Only the discounted value of each path leaves the kernel; a
// second kernel reduces those in a fixed order (bitwise reproducible).
//
// Scheduling: a persistent grid; each warp takes (contract, path-range) work
// items from an atomic counter and its 32 lanes take paths one by one from
// the item. A lane whose path is finished early (every flow emitted or knocked
// out) starts a new path at once, so knocked-out barrier paths do not hold a
// lane idle. Path-to-lane assignment depends only on the data, and per-path
// values are written to fixed slots, so results do not depend on timing.
#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>

#include "device_common.cuh"
#include "engine.hpp"
#include "ffloat.cuh"
#include "launch.hpp"
#include "stats.cuh"

namespace kx {

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        raise(KX_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

void DevBuf::ensure(size_t bytes) {
    if (bytes <= cap) return;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes, 256);
    KX_CUDA(cudaMalloc(&p, want));
    cap = want;
}

void PinnedBuf::ensure(size_t bytes) {
    if (bytes <= cap) return;
    const size_t want = std::max<size_t>(std::max<size_t>(bytes, 4096), 2 * cap);  // grow geometrically
    if (p) cudaFreeHost(p);  // the previous call's copies completed before it returned
    p = nullptr;
    cap = 0;
    KX_CUDA(cudaHostAlloc(&p, want, cudaHostAllocDefault));
    cap = want;
}

Ctx &ctx() {
    static Ctx c;
    static std::mutex setup_mu;
    if (c.ready.load(std::memory_order_acquire)) return c;
    std::lock_guard<std::mutex> g(setup_mu);
    if (c.ready.load(std::memory_order_relaxed)) return c;  // another thread finished the set-up
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= 0) {
        cudaGetLastError();
        raise(KX_NO_DEVICE, std::string("no CUDA device: ") + (e == cudaSuccess ? "count is 0" : cudaGetErrorString(e)));
    }
    KX_CUDA(cudaSetDevice(c.device));
    cudaDeviceProp prop;
    KX_CUDA(cudaGetDeviceProperties(&prop, c.device));
    c.sm_count = prop.multiProcessorCount;
    c.cc_major = prop.major;
    c.cc_minor = prop.minor;
    c.name = prop.name;
    // a set-up that failed half way is retried by the next call: keep what exists
    if (!c.stream) KX_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    if (!c.ev0) KX_CUDA(cudaEventCreate(&c.ev0));
    if (!c.ev1) KX_CUDA(cudaEventCreate(&c.ev1));
    c.ready.store(true, std::memory_order_release);
    return c;
}

int persistent_blocks(const void *kernel, int block, size_t smem) {
    Ctx &c = ctx();
    int per_sm = 0;
    KX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem));
    if (per_sm < 1) raise(KX_CUDA_ERROR, "kernel does not fit on an SM");
    return per_sm * c.sm_count;
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------
// Deterministic chunk statistics: each cluster of blocks takes one fixed chunk
// of values and returns (n, mean, M2) from exact integer sums
// (pricer.rs:303-328 takes two passes over the values; the integer sums give
// its mean and M2 with one or two roundings): prices (k_chunk_stats_exact) and
// estimators sum_s w[s] * vals[s * stride + i] formed per path in FP64
// (k_chunk_stats: Greek estimators, variance-reduction corrections,
// multilevel differences with w = {1, -1}).
// ---------------------------------------------------------------------------
__global__ void __cluster_dims__(KX_STATS_CLUSTER, 1, 1) __launch_bounds__(KX_STATS_THREADS, 4)
    k_chunk_stats_exact(const double *__restrict__ vals, const ChunkDesc *__restrict__ ch, ChunkOut *__restrict__ out) {
    __shared__ uint32_t emax[KX_STATS_THREADS / 32 + KX_STATS_CLUSTER];
    __shared__ uint64_t part[4 * (KX_STATS_THREADS / 32 + KX_STATS_CLUSTER)];
    __shared__ double red[32];
    const uint32_t q = blockIdx.x / KX_STATS_CLUSTER;  // the chunk of this cluster
    const ChunkDesc c = ch[q];
    const double *v = vals + c.begin;
    double mean = 0.0, m2 = 0.0;
    chunk_moments_exact_cluster<KX_STATS_CLUSTER, KX_STATS_THREADS>([&](uint32_t i) { return v[i]; }, c.count, emax,
                                                                     part, red, mean, m2);
    if (blockIdx.x % KX_STATS_CLUSTER == 0 && threadIdx.x == 0) out[q] = ChunkOut{(double)c.count, mean, m2};
}

// NS: the scenario count when it is 2 (multilevel differences, two-point
// estimators: the loads of a value unrolled and issued together), 0 for any
// count ns <= 8. 3 blocks per SM: the scenario operands take registers.
template <int NS>
__global__ void __cluster_dims__(KX_STATS_CLUSTER, 1, 1) __launch_bounds__(KX_STATS_THREADS, 3)
    k_chunk_stats(const double *__restrict__ vals, uint64_t stride, int ns, const double *__restrict__ w,
                  const ChunkDesc *__restrict__ ch, ChunkOut *__restrict__ out) {
    __shared__ uint32_t emax[KX_STATS_THREADS / 32 + KX_STATS_CLUSTER];
    __shared__ uint64_t part[4 * (KX_STATS_THREADS / 32 + KX_STATS_CLUSTER)];
    __shared__ double red[32];
    __shared__ double ww[8];
    if (threadIdx.x < 8) ww[threadIdx.x] = (int)threadIdx.x < ns ? w[threadIdx.x] : 0.0;
    __syncthreads();
    const uint32_t q = blockIdx.x / KX_STATS_CLUSTER;
    const ChunkDesc c = ch[q];
    const double *v = vals + c.begin;
    double mean = 0.0, m2 = 0.0;
    chunk_moments_exact_cluster<KX_STATS_CLUSTER, KX_STATS_THREADS>(
        [&](uint32_t i) {
            double x = ww[0] * v[i];
            if (NS > 0) {
#pragma unroll
                for (int s = 1; s < NS; ++s) x = fma(ww[s], v[(uint64_t)s * stride + i], x);
            } else {
                for (int s = 1; s < ns; ++s) x = fma(ww[s], v[(uint64_t)s * stride + i], x);
            }
            return x;
        },
        c.count, emax, part, red, mean, m2);
    if (blockIdx.x % KX_STATS_CLUSTER == 0 && threadIdx.x == 0) out[q] = ChunkOut{(double)c.count, mean, m2};
}

// The same statistics in compensated FP32 (KX_PREC_FP32_KAHAN): each path's
// value is rounded to FP32 once; every thread adds its values with Kahan's
// compensated summation (the sum and its running correction), the threads'
// (sum, correction) pairs are added in float-float in a fixed tree, and the
// chunk's mean and M2 leave as doubles for the final cross-chunk merge, the
// only FP64 arithmetic of the call's reduction.
__device__ __forceinline__ ff ff_block_sum(ff v, ff *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = ff_add(v, ff{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    ff t = ff{0.0f, 0.0f};
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : ff{0.0f, 0.0f};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = ff_add(t, ff{__shfl_xor_sync(0xffffffffu, t.hi, o), __shfl_xor_sync(0xffffffffu, t.lo, o)});
    }
    __syncthreads();
    if (threadIdx.x == 0) red[0] = t;
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(256) k_chunk_stats_kahan(const double *__restrict__ vals,
                                                           const ChunkDesc *__restrict__ ch, ChunkOut *__restrict__ out) {
    __shared__ ff red[32];
    const ChunkDesc c = ch[blockIdx.x];
    float s = 0.0f, e = 0.0f;  // Kahan: running sum and the correction of its lost low part
    for (uint32_t i = threadIdx.x; i < c.count; i += blockDim.x) {
        const float x = __fsub_rn((float)vals[c.begin + i], e);
        const float t = __fadd_rn(s, x);
        e = __fsub_rn(__fsub_rn(t, s), x);
        s = t;
    }
    const ff sum = ff_block_sum(ff{s, -e}, red);
    const ff mean = ff_div(sum, ff_make((float)c.count));
    float q = 0.0f, f = 0.0f;
    for (uint32_t i = threadIdx.x; i < c.count; i += blockDim.x) {
        const ff dv = ff_sub(ff_make((float)vals[c.begin + i]), mean);
        const ff d2 = ff_mul(dv, dv);
        const float x = __fsub_rn(d2.hi, f);
        const float t = __fadd_rn(q, x);
        f = __fsub_rn(__fsub_rn(t, q), x);
        q = t;
    }
    const ff m2 = ff_block_sum(ff{q, -f}, red);
    if (threadIdx.x == 0)
        out[blockIdx.x] = ChunkOut{(double)c.count, (double)mean.hi + (double)mean.lo, (double)m2.hi + (double)m2.lo};
}

std::vector<Stats> device_stats(Ctx &c, const double *values, uint64_t stride, const std::vector<StatsJob> &jobs) {
    const uint32_t CH = KX_STATS_CHUNK;
    std::vector<ChunkDesc> chunks;
    std::vector<size_t> first(jobs.size() + 1, 0);
    for (size_t j = 0; j < jobs.size(); ++j) {
        first[j] = chunks.size();
        for (uint64_t b = 0; b < jobs[j].n; b += CH)
            chunks.push_back(ChunkDesc{jobs[j].begin + b, (uint32_t)std::min<uint64_t>(CH, jobs[j].n - b), 0});
    }
    first[jobs.size()] = chunks.size();
    std::vector<Stats> res(jobs.size());
    if (chunks.empty()) return res;
    // jobs with different weights run as separate launches; the chunk table and the weights go
    // up in one copy from pinned memory, the chunks' statistics come back the same way
    const size_t b_chunks = chunks.size() * sizeof(ChunkDesc), b_w = jobs.size() * 8 * sizeof(double);
    const size_t b_out = chunks.size() * sizeof(ChunkOut);
    c.stats_in.ensure(b_chunks + b_w);
    c.chunk_out.ensure(b_out);
    c.stats_stage.ensure(std::max(b_chunks + b_w, b_out));
    unsigned char *stage = c.stats_stage.as<unsigned char>();
    memcpy(stage, chunks.data(), b_chunks);
    double *wts = reinterpret_cast<double *>(stage + b_chunks);
    for (size_t j = 0; j < jobs.size(); ++j)
        for (int s = 0; s < 8; ++s) wts[j * 8 + s] = jobs[j].w[s];
    KX_CUDA(cudaMemcpyAsync(c.stats_in.p, stage, b_chunks + b_w, cudaMemcpyHostToDevice, c.stream));
    const ChunkDesc *d_chunks = c.stats_in.as<ChunkDesc>();
    const double *d_w = reinterpret_cast<const double *>(c.stats_in.as<unsigned char>() + b_chunks);
    KX_CUDA(cudaEventRecord(c.ev0, c.stream));
    // one launch per run of consecutive jobs with the same weights
    for (size_t j = 0; j < jobs.size();) {
        size_t e = j + 1;
        while (e < jobs.size() && jobs[e].ns == jobs[j].ns && !memcmp(jobs[e].w, jobs[j].w, sizeof jobs[j].w)) ++e;
        const size_t nc = first[e] - first[j];
        const bool plain = jobs[j].ns == 1 && jobs[j].w[0] == 1.0;
        if (nc && c.kahan_stats && plain) {  // KX_PREC_FP32_KAHAN: compensated FP32 sums
            k_chunk_stats_kahan<<<(unsigned)nc, 256, 0, c.stream>>>(values, d_chunks + first[j],
                                                                    c.chunk_out.as<ChunkOut>() + first[j]);
            KX_CUDA(cudaGetLastError());
            c.last.kernel_launches++;
        } else if (nc && plain) {
            k_chunk_stats_exact<<<(unsigned)nc * KX_STATS_CLUSTER, KX_STATS_THREADS, 0, c.stream>>>(
                values, d_chunks + first[j], c.chunk_out.as<ChunkOut>() + first[j]);
            KX_CUDA(cudaGetLastError());
            c.last.kernel_launches++;
        } else if (nc) {  // weighted scenarios, multilevel differences
            const int ns = jobs[j].ns;
            auto kfn = ns == 2 ? k_chunk_stats<2> : k_chunk_stats<0>;
            kfn<<<(unsigned)nc * KX_STATS_CLUSTER, KX_STATS_THREADS, 0, c.stream>>>(
                values, stride, ns, d_w + j * 8, d_chunks + first[j], c.chunk_out.as<ChunkOut>() + first[j]);
            KX_CUDA(cudaGetLastError());
            c.last.kernel_launches++;
        }
        j = e;
    }
    KX_CUDA(cudaEventRecord(c.ev1, c.stream));
    const ChunkOut *h = c.stats_stage.as<ChunkOut>();  // the staged uploads were consumed in stream order
    KX_CUDA(cudaMemcpyAsync(c.stats_stage.p, c.chunk_out.p, b_out, cudaMemcpyDeviceToHost, c.stream));
    KX_CUDA(cudaStreamSynchronize(c.stream));
    float rms = 0.f;
    KX_CUDA(cudaEventElapsedTime(&rms, c.ev0, c.ev1));
    c.last.reduce_ms += rms;
    c.last.d2h_bytes += b_out;
    for (size_t j = 0; j < jobs.size(); ++j) res[j] = merge_chunks(h + first[j], first[j + 1] - first[j]);
    return res;
}

Stats merge_chunks(const ChunkOut *h, size_t n) {
    Stats s;
    for (size_t q = 0; q < n; ++q) {  // Chan et al. pairwise merge, fixed order
        const ChunkOut &o = h[q];
        if (s.n == 0) { s.n = o.n; s.mean = o.mean; s.m2 = o.m2; continue; }
        const double tn = s.n + o.n;
        if (o.mean == s.mean) {  // d = 0: the same result, and equal infinite means stay infinite
            s.m2 = s.m2 + o.m2;  // (as the reference's one-pass mean, pricer.rs:303-328)
        } else {
            const double d = o.mean - s.mean;
            s.mean = s.mean + d * (o.n / tn);
            s.m2 = s.m2 + o.m2 + d * d * (s.n * o.n / tn);
        }
        s.n = tn;
    }
    return s;
}

void launch_chunk_stats(cudaStream_t s, const double *values, const ChunkDesc *chunks, ChunkOut *out,
                        unsigned n_chunks) {
    if (!n_chunks) return;
    k_chunk_stats_exact<<<n_chunks * KX_STATS_CLUSTER, KX_STATS_THREADS, 0, s>>>(values, chunks, out);
    KX_CUDA(cudaGetLastError());
}

kx_price_result finish(const Stats &s) {  // pricer.rs:303-328
    const double Z95 = 1.959963984540054;
    kx_price_result r{};
    const uint64_t n = (uint64_t)s.n;
    r.price = n ? s.mean : 0.0;
    r.sample_std = n > 1 ? std::sqrt(s.m2 / ((double)n - 1.0)) : 0.0;
    r.std_error = n > 0 ? r.sample_std / std::sqrt((double)n) : 0.0;
    r.ci95_low = r.price - Z95 * r.std_error;
    r.ci95_high = r.price + Z95 * r.std_error;
    r.n_paths = n;
    return r;
}

// ---------------------------------------------------------------------------
// host side of a path launch
// ---------------------------------------------------------------------------
void check_cfg(const kx_mc_config *cfg) {
    if (!cfg) raise(KX_INVALID_ARGUMENT, "config is NULL");
    if (cfg->rng != KX_RNG_PHILOX && cfg->rng != KX_RNG_SHARED_DRAWS) raise(KX_INVALID_ARGUMENT, "unknown rng");
    if (cfg->precision != KX_PREC_FP32 && cfg->precision != KX_PREC_FP64 && cfg->precision != KX_PREC_FP32_KAHAN)
        raise(KX_INVALID_ARGUMENT, "unknown precision");
    if (cfg->flags != 0) raise(KX_INVALID_ARGUMENT, "flags must be 0");
    if (cfg->n_paths >= (1ull << 32)) raise(KX_INVALID_ARGUMENT, "n_paths must be below 2^32");
}

Job make_job(const Program &p, const Model &m, const kx_mc_config &cfg, const std::vector<double> &grid,
             const std::vector<Scenario> &scen_in, int smooth, double smooth_w) {
    Job j;
    j.model = m;
    validate_model(m);
    validate_grid(grid);
    std::vector<Scenario> scen = scen_in;
    if (m.kind == KX_MODEL_MULTI_GBM) {  // factor i in the per-scenario slots i (M_MULTI)
        scen.clear();
        for (size_t i = 0; i < m.assets.size(); ++i) scen.push_back(Scenario{m.a_s0[i], m.a_mu[i], m.a_sigma[i], cfg.rate});
    }
    if (scen.empty()) scen.push_back(Scenario{m.s0, m.mu, m.sigma, cfg.rate});
    const int ns = (int)scen.size();
    Model m0 = m;
    m0.s0 = scen[0].s0;
    m0.mu = scen[0].mu;
    m0.sigma = scen[0].sigma;
    bind(p.low, grid, m0, scen[0].rate, j.prog, j.tab);
    const size_t n = grid.size();
    if (ns > 1) {  // bump scenarios step with dt / sqrt(dt) and their own drift and volatility
        for (size_t k = 0; k < n; ++k) {
            const double dt = k == 0 ? grid[0] : grid[k] - grid[k - 1];
            j.tab.c0[k] = dt;
            j.tab.c1[k] = std::sqrt(dt);
        }
        j.tab.disc.resize(n * ns);
        for (int s = 0; s < ns; ++s)
            for (size_t k = 0; k < n; ++k) j.tab.disc[s * n + k] = std::exp(-scen[s].rate * grid[k]);
    }
    // log-spot thresholds of Spot-cmp-Const conditions, per scenario
    bool nonpos = false;
    for (auto &sc : scen) nonpos |= !(sc.s0 > 0.0);
    if (nonpos) {  // log-space compare impossible: evaluate those conditions in full
        for (int i = 0; i < j.prog.n_trig; ++i)
            if (j.prog.trig[i].cond_kind == CK_SPOT_CMP) j.prog.trig[i].cond_kind = CK_GENERAL;
        j.prog.spot_each_step = 1;
    }
    j.thr.assign((size_t)KX_MAX_NS * KX_MAX_SPOT, 0.0);
    for (int s = 0; s < KX_MAX_NS; ++s) {
        const Scenario &sc = scen[std::min(s, ns - 1)];
        for (size_t q = 0; q < p.low.spot_cmp.size() && q < (size_t)KX_MAX_SPOT; ++q)
            if (sc.s0 > 0.0) j.thr[(size_t)s * KX_MAX_SPOT + q] = std::log(p.low.spot_cmp[q].c / sc.s0);
    }
    ContractDev &d = j.dev;
    memset(&d, 0, sizeof d);
    d.n_times = (int32_t)n;
    d.n_paths = cfg.n_paths;
    d.seed = cfg.seed;
    d.stream = 0;
    d.smooth = smooth;
    d.heston_scheme = m.scheme;
    for (int s = 0; s < KX_MAX_NS; ++s) {
        const Scenario &sc = scen[std::min(s, ns - 1)];
        d.s0[s] = sc.s0;
        d.drift[s] = sc.mu - 0.5 * sc.sigma * sc.sigma;
        d.sigma[s] = sc.sigma;
        d.s0f[s] = (float)d.s0[s];
        d.driftf[s] = (float)d.drift[s];
        d.sigmaf[s] = (float)d.sigma[s];
    }
    if (m.kind == KX_MODEL_MULTI_GBM) {
        d.n_assets = (int32_t)m.assets.size();
        for (size_t q = 0; q < m.chol.size(); ++q) {
            d.chol[q] = m.chol[q];
            d.cholf[q] = (float)m.chol[q];
        }
    }
    d.v0 = m.v0; d.kappa = m.kappa; d.theta = m.theta; d.sigma_v = m.sigma_v; d.rho = m.rho;
    d.rho_perp = std::sqrt(std::max(1.0 - m.rho * m.rho, 0.0));  // simulator.rs:510
    d.r = m.r;
    d.inv_w = smooth ? 1.0 / smooth_w : 0.0;
    // uniform grid: every step's coefficients equal in the launch precision
    d.uniform = 0;
    if (n > 1) {
        bool uni = true;
        for (size_t k = 2; k < n && uni; ++k) {
            if (cfg.precision == KX_PREC_FP64) uni = j.tab.c0[k] == j.tab.c0[1] && j.tab.c1[k] == j.tab.c1[1];
            else uni = (float)j.tab.c0[k] == (float)j.tab.c0[1] && (float)j.tab.c1[k] == (float)j.tab.c1[1];
        }
        d.uniform = uni ? 1 : 0;
        d.uc0 = j.tab.c0[1];
        d.uc1 = j.tab.c1[1];
        d.uc0f = (float)d.uc0;
        d.uc1f = (float)d.uc1;
    }
    d.v0f = (float)d.v0; d.kappaf = (float)d.kappa; d.thetaf = (float)d.theta; d.sigma_vf = (float)d.sigma_v;
    d.rhof = (float)d.rho; d.rho_perpf = (float)d.rho_perp; d.rf = (float)d.r; d.inv_wf = (float)d.inv_w;
    return j;
}

template <class Real>
void pack_steps(const StepTables &t, std::vector<unsigned char> &out) {
    const size_t n = t.c0.size();
    const size_t off = out.size();
    out.resize(off + n * sizeof(StepRec<Real>));
    StepRec<Real> *r = reinterpret_cast<StepRec<Real> *>(out.data() + off);
    for (size_t k = 0; k < n; ++k) r[k] = StepRec<Real>{(Real)t.c0[k], (Real)t.c1[k], t.time_true[k], 0u};
}
template void pack_steps<float>(const StepTables &, std::vector<unsigned char> &);
template void pack_steps<double>(const StepTables &, std::vector<unsigned char> &);

// Launch the fused path kernel over `jobs` (all of one model kind, one
// precision and one scenario count). Per-path values land in c.pv:
// scenario s of job j, path i at s * stride + jobs[j].dev.pv_off + i.
const void *select_kernel(int model, bool f64, int ns, int minb, bool lean, bool stat, bool acc, bool sm) {
    if (model == KX_MODEL_MULTI_GBM) return paths_kernel_multi(f64, minb);  // general handler
    if (lean) {
        if (sm && model != KX_MODEL_GBM) return nullptr;
        return model == KX_MODEL_GBM ? lean_kernel_gbm(f64, minb, stat, acc, sm)
                                     : lean_kernel_heston(f64, minb, stat, acc);
    }
    if (ns != 1) raise(KX_CUDA_ERROR, "path launches carry one scenario");
    return model == KX_MODEL_GBM ? paths_kernel_gbm(f64, minb) : paths_kernel_heston(f64, minb);
}

// k_lean serves launches whose contracts test the price only through
// Spot-cmp-Const conditions and keep no averages or extrema (one scenario,
// no smoothing). Both kernels value every path identically; KX_PATH_KERNEL
// = "general" or "lean" forces one of them (the lean one only where it applies).
// A contract's one accumulator of the spot that the static family of k_lean
// keeps in registers: an average over a window, a running max or min (no
// nesting).
static bool lean_average(const KxProgram &P) {
    return P.n_acc == 1 && P.acc[0].inner == IK_SPOT && !P.acc[0].static_err;
}

// until(Spot cmp Const) slots that a smoothed job weighs instead of knocking.
static int smoothed_untils(const Job &j) {
    if (!j.dev.smooth) return 0;
    int n = 0;
    for (int i = 0; i < j.prog.n_trig; ++i)
        n += j.prog.trig[i].kind == TK_UNTIL && j.prog.trig[i].cond_kind == CK_SPOT_CMP;
    return n;
}

bool lean_smoothed(const std::vector<Job> &jobs) {
    for (auto &j : jobs)
        if (smoothed_untils(j)) return true;
    return false;
}

static bool lean_applies(const std::vector<Job> &jobs, int ns) {
    if (ns != 1) return false;
    bool avg = false;
    const bool sm = lean_smoothed(jobs);
    for (auto &j : jobs) {
        if (j.model.kind == KX_MODEL_MULTI_GBM) return false;
        if (sm) {  // smoothed barriers: GBM on static schedules (survival weights in registers)
            StaticDev T;
            if (j.model.kind != KX_MODEL_GBM || j.prog.n_acc || !build_static(j, T)) return false;
        }
        if (j.prog.n_acc && !lean_average(j.prog)) return false;
        // the spot each step: for the average (kept by k_lean) or a general condition (not served)
        if (j.prog.spot_each_step && !j.prog.n_acc) return false;
        avg = avg || j.prog.n_acc;
        for (int i = 0; i < j.prog.n_trig; ++i)
            if (j.prog.trig[i].cond_kind == CK_GENERAL) return false;
    }
    if (avg) {  // averages only on static schedules
        StaticDev T;
        for (auto &j : jobs)
            if (!build_static(j, T)) return false;
    }
    return true;
}

bool lean_has_average(const std::vector<Job> &jobs) {
    for (auto &j : jobs)
        if (j.prog.n_acc) return true;
    return false;
}

bool use_lean(const std::vector<Job> &jobs, int ns) {
    const char *env = getenv("KX_PATH_KERNEL");
    if (env && strcmp(env, "general") == 0) return false;
    // "lean" forces the general event handler, which keeps no averages and weighs no barrier
    if (env && strcmp(env, "lean") == 0 && (lean_has_average(jobs) || lean_smoothed(jobs))) return false;
    return lean_applies(jobs, ns);
}

// The static schedule of a lean job (StaticDev), or false when the contract
// has none: a when/anytime reading prices, an amount without closed form,
// an error-capable evaluation, or more than KX_MAX_SEV event steps.
bool build_static(const Job &j, StaticDev &T) {
    const KxProgram &P = j.prog;
    if (P.n_acc > 1 || (P.n_acc == 1 && !lean_average(P))) return false;
    // amounts without a closed form only when they read the average (the interpreter evaluates them)
    if (!P.n_acc && (P.err_capable || (P.all_leaves & ~P.simple_leaves) != 0u)) return false;
    const StaticSchedule S = static_schedule(P, j.tab);
    if (!S.static_ok) return false;
    // an average can only fail when read too early (acc_value): every flow that reads it pays at a
    // known step, so the schedule is error-free when each such step is at or after its first valid one
    if (P.n_acc)
        for (auto &f : S.flows)
            if (P.leaf[f.leaf].err_capable && f.step < P.acc[0].e_min) return false;
    memset(&T, 0, sizeof T);
    std::map<int, std::pair<uint32_t, uint32_t>> at;  // step -> (armed barriers, paid flows)
    for (auto &f : S.flows) {
        at[f.step].second |= 1u << f.leaf;
        T.all_flows |= 1u << f.leaf;
        for (int i = 0; i < P.n_trig; ++i)
            if ((f.price_untils >> i) & 1u) T.kill[i] |= 1u << f.leaf;
    }
    const bool smooth = j.dev.smooth != 0;
    int sm_spot[KX_MAX_SM] = {-1, -1};
    for (int i = 0; i < P.n_trig; ++i) {
        const KxTrig &Tr = P.trig[i];
        if (Tr.cond_kind == CK_GENERAL) return false;
        if (Tr.cond_kind != CK_SPOT_CMP) continue;
        if (Tr.kind != TK_UNTIL) return false;
        if (S.arm[i] == StaticSchedule::NEVER || T.kill[i] == 0u) continue;  // never tested, or drops nothing
        if (smooth) {  // weighs instead of knocking: no arming event, not a live barrier
            if (P.n_acc || T.n_sm >= KX_MAX_SM) return false;
            for (int q = 0; q < T.n_sm; ++q)
                if (sm_spot[q] == Tr.spot_slot) return false;  // one weight per condition slot (as on_event)
            const int q = T.n_sm++;
            sm_spot[q] = Tr.spot_slot;
            const double t = j.thr[Tr.spot_slot];
            const bool down = Tr.cmp == CMP_LE || Tr.cmp == CMP_LT;
            T.sm_arm[q] = S.arm[i];
            T.sm_flows[q] = T.kill[i];
            T.sm_thr64[q] = t;
            T.sm_thr32[q] = (float)t;
            T.sm_mul64[q] = down ? -j.dev.inv_w : j.dev.inv_w;  // (y - t) * -m is exactly -((y - t) * m)
            T.sm_mul32[q] = down ? -j.dev.inv_wf : j.dev.inv_wf;
            continue;
        }
        at[S.arm[i]].first |= 1u << i;
        const double t = j.thr[Tr.spot_slot];
        const float tf = (float)t;
        const bool up = Tr.cmp == CMP_GE || Tr.cmp == CMP_GT;
        if (up) T.up_mask |= 1u << i;
        switch (Tr.cmp) {  // strict comparisons become inclusive at the next representable threshold
        case CMP_GT: T.thr64[i] = std::nextafter(t, INFINITY); T.thr32[i] = std::nextafter(tf, INFINITY); break;
        case CMP_LT: T.thr64[i] = std::nextafter(t, -INFINITY); T.thr32[i] = std::nextafter(tf, -INFINITY); break;
        default: T.thr64[i] = t; T.thr32[i] = tf; break;
        }
    }
    if (at.size() > (size_t)KX_MAX_SEV) return false;
    for (auto &kv : at) {
        T.ev_step[T.n_ev] = kv.first;
        T.ev_arm[T.n_ev] = kv.second.first;
        T.ev_pay[T.n_ev] = kv.second.second;
        ++T.n_ev;
    }
    for (int q = 0; q < P.n_leaf; ++q) {
        const KxLeaf &F = P.leaf[q];
        const bool simple = (P.simple_leaves >> q) & 1u;
        T.f_fast[q] = F.kind == AK_CONST || !simple ? (uint8_t)FA_NONE : F.fast;
        T.f_k[q] = F.kind == AK_CONST || !simple ? 0.0 : P.cpool[F.fast_k];
        T.f_sign[q] = F.sign;
        if (F.sign < 0.0) T.f_neg |= 1u << q;
        if (F.kind != AK_CONST && !simple) T.gen_flows |= 1u << q;
    }
    if (P.n_acc) {
        T.acc_on = 1;
        T.acc_from = P.acc[0].i_from;
        T.acc_to = P.acc[0].i_to;
        T.acc_kind = P.acc[0].kind;
    }
    return true;
}

// Static schedules serve a lean launch whose every contract has one, unless
// KX_PATH_KERNEL = "lean" asks for the general event handler.
bool use_static(const std::vector<Job> &jobs, int ns) {
    if (!use_lean(jobs, ns)) return false;
    const char *env = getenv("KX_PATH_KERNEL");
    if (env && strcmp(env, "lean") == 0) return false;
    StaticDev T;
    for (auto &j : jobs)
        if (!build_static(j, T)) return false;
    return true;
}

static uint64_t run_paths_v(Ctx &c, std::vector<Job> &jobs, const kx_mc_config &cfg, int ns, uint64_t &stride_out,
                            int minb, bool lean, bool pair = false);

// Project autotuner: the path kernel exists at a few register budgets
// (minimum resident blocks per SM). The first launch of each kind (model,
// precision, scenario count, program features) times every variant on a
// calibration batch of the same contracts and keeps the fastest. All variants
// compute every path identically, so the choice never changes results.
// KX_TUNE=0 disables tuning (the default budget is used).
struct TuneEntry {
    int minb;
    float ms[8];
};
static std::map<std::string, TuneEntry> g_tune;

static std::string tune_key(const std::vector<Job> &jobs, const kx_mc_config &cfg, int ns) {
    int acc = 0, gen = 0, smooth = 0, spot = 0;
    for (auto &j : jobs) {
        acc = std::max(acc, j.prog.n_acc);
        spot |= j.prog.spot_each_step ? 1 : 0;
        smooth |= j.dev.smooth;
        for (int i = 0; i < j.prog.n_trig; ++i) gen |= j.prog.trig[i].cond_kind == CK_GENERAL;
    }
    char buf[128];
    snprintf(buf, sizeof buf, "m%d-p%d-ns%d-acc%d-gen%d-sm%d-sp%d-l%d", jobs[0].model.kind, cfg.precision, ns, acc > 0,
             gen, smooth, spot, use_static(jobs, ns) ? 2 : use_lean(jobs, ns) ? 1 : 0);
    return buf;
}

const int *variants(int model, bool f64, int ns, bool lean, int &n) {
    static const int vm32[] = {4, 3, 2};
    static const int vm64[] = {2};
    if (model == KX_MODEL_MULTI_GBM) {  // the budgets of paths_multi.cu
        n = f64 ? 1 : 3;
        return f64 ? vm64 : vm32;
    }
    static const int v1[] = {4, 3, 2};
    static const int l32[] = {4, 5, 6};
    static const int lg32[] = {4, 5, 6, 3};  // GBM: 3 blocks per SM keeps the accumulator family unspilled
    static const int lg64[] = {4, 3};
    static const int lh64[] = {3};
    if (lean) {
        if (!f64 && model == KX_MODEL_GBM) { n = 4; return lg32; }
        if (!f64) { n = 3; return l32; }
        if (model == KX_MODEL_GBM) { n = 2; return lg64; }
        n = 1;
        return lh64;
    }
    (void)ns;
    n = 3;
    return v1;
}

static uint64_t run_paths(Ctx &c, std::vector<Job> &jobs, const kx_mc_config &cfg, int ns, uint64_t &stride_out) {
    int nv = 0;
    const bool lean = use_lean(jobs, ns);
    const int *vs = variants(jobs[0].model.kind, cfg.precision == KX_PREC_FP64, ns, lean, nv);
    const char *env = getenv("KX_TUNE");
    const bool tune = !(env && env[0] == '0');
    const std::string key = tune_key(jobs, cfg, ns);
    auto it = g_tune.find(key);
    if (tune && nv > 1 && it == g_tune.end()) {
        // calibration batch: the same contracts with fewer paths
        uint64_t total = 0;
        for (auto &j : jobs) total += j.dev.n_paths;
        if (total >= (1u << 16)) {
            std::vector<Job> cal = jobs;
            const double scale = std::min(1.0, (double)(1u << 20) / (double)total);
            for (auto &j : cal) j.dev.n_paths = std::max<uint64_t>(1, (uint64_t)(j.dev.n_paths * scale));
            const kx_launch_stats saved = c.last;
            TuneEntry e{};
            float best = 1e30f;
            for (int q = 0; q < nv; ++q) {
                float t = 1e30f;
                for (int rep = 0; rep < 2; ++rep) {
                    c.last.kernel_ms = 0;
                    uint64_t st = 0;
                    run_paths_v(c, cal, cfg, ns, st, vs[q], lean);
                    t = std::min(t, (float)c.last.kernel_ms);
                }
                e.ms[q] = t;
                if (t < best) { best = t; e.minb = vs[q]; }
            }
            c.last = saved;
            it = g_tune.emplace(key, e).first;
            const char *vb = getenv("KX_TUNE_VERBOSE");
            if (vb && vb[0] == '1') {
                fprintf(stderr, "[kx tune] %s:", key.c_str());
                for (int q = 0; q < nv; ++q) fprintf(stderr, " minb%d=%.3fms", vs[q], e.ms[q]);
                fprintf(stderr, " -> minb%d\n", e.minb);
            }
        }
    }
    const int minb = it != g_tune.end() ? it->second.minb : vs[0];
    return run_paths_v(c, jobs, cfg, ns, stride_out, minb, lean);
}

PathPlan plan_paths(std::vector<Job> &jobs, const kx_mc_config &cfg, int ns, int minb, bool lean,
                    uint64_t item_paths, bool stat, bool pair) {
    PathPlan P;
    P.f64 = cfg.precision == KX_PREC_FP64;
    P.lean = lean;
    P.stat = lean && stat;
    P.acc = P.stat && lean_has_average(jobs);
    P.sm = P.stat && lean_smoothed(jobs);
    if (lean && !P.stat && lean_has_average(jobs)) raise(KX_CUDA_ERROR, "averages need the static family");
    if (lean && !P.stat && lean_smoothed(jobs)) raise(KX_CUDA_ERROR, "smoothed barriers need the static family");
    if (P.stat) {
        P.statics.resize(jobs.size());
        for (size_t q = 0; q < jobs.size(); ++q)
            if (!build_static(jobs[q], P.statics[q])) raise(KX_CUDA_ERROR, "static schedule expected");
    }
    P.model = jobs[0].model.kind;
    P.ns = ns;
    P.minb = minb;
    const bool f64 = P.f64;
    int max_spot = 0, max_acc = 0;
    for (auto &j : jobs) {
        ContractDev d = j.dev;
        d.prog = (int32_t)P.progs.size();
        P.progs.push_back(j.prog);
        d.step_off = (int32_t)(P.steps.size() / (f64 ? sizeof(StepRec<double>) : sizeof(StepRec<float>)));
        if (f64) pack_steps<double>(j.tab, P.steps);
        else pack_steps<float>(j.tab, P.steps);
        d.disc_off = (int32_t)P.disc.size();
        P.disc.insert(P.disc.end(), j.tab.disc.begin(), j.tab.disc.end());
        // per-path values of paths path_base .. path_base + n - 1 land at
        // pv_off .. pv_off + n - 1: the kernels index pv_off + path (mod 2^64)
        d.pv_off = P.total - (uint64_t)j.path_base;
        j.dev.pv_off = P.total;
        P.total += d.n_paths;
        P.path_steps += d.n_paths * (uint64_t)(d.n_times > 0 ? d.n_times - 1 : 0);
        max_spot = std::max(max_spot, j.prog.n_spot_cmp);
        max_acc = std::max(max_acc, j.prog.n_acc);
        const size_t toff = P.thr.size();
        if (f64) {
            P.thr.resize(toff + j.thr.size() * sizeof(double));
            memcpy(P.thr.data() + toff, j.thr.data(), j.thr.size() * sizeof(double));
        } else {
            P.thr.resize(toff + j.thr.size() * sizeof(float));
            float *t = reinterpret_cast<float *>(P.thr.data() + toff);
            for (size_t q = 0; q < j.thr.size(); ++q) t[q] = (float)j.thr[q];
        }
        P.cons.push_back(d);
    }
    // work items: contiguous per contract, costliest contracts first
    std::vector<int> order(jobs.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return P.cons[a].n_paths * (uint64_t)P.cons[a].n_times > P.cons[b].n_paths * (uint64_t)P.cons[b].n_times;
    });
    const int block = KX_BLOCK;
    const bool smooth = jobs[0].dev.smooth != 0;
    P.surv_base = 2u * (uint32_t)max_acc;
    P.slots = P.surv_base + (smooth ? (uint32_t)max_spot : 0u);
    P.smem = lean ? 0 : (size_t)ns * P.slots * block * (f64 ? 8 : 4);  // k_lean keeps its average in registers
    if (pair && P.sm) raise(KX_UNSUPPORTED, "smoothed barriers on multilevel pairs");
    P.kfn = !pair ? select_kernel(P.model, f64, ns, minb, lean, P.stat, P.acc, P.sm)
            : lean ? lean_kernel_pair(P.model, f64, P.stat, P.acc)
                   : paths_kernel_pair(P.model, f64);
    if (!P.kfn) raise(KX_CUDA_ERROR, "missing kernel variant");
    if (P.smem > 48 * 1024)
        KX_CUDA(cudaFuncSetAttribute(P.kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem));
    const int full = persistent_blocks(P.kfn, block, P.smem);
    const uint64_t warps_total = (uint64_t)full * (block / 32);
    uint64_t item = item_paths;
    if (item == 0) {  // about 8 items per warp, 64..2048 paths each
        item = P.total / std::max<uint64_t>(1, warps_total * 8);
        item = std::max<uint64_t>(64, std::min<uint64_t>(2048, item));
    }
    item = (item + 31) / 32 * 32;
    P.item_paths = item;
    // arithmetic items: per contract in launch order, its item count. A
    // one-contract launch ends in items of 32 paths (a path per lane), about
    // one such item per resident warp: when the queue runs dry the warps hold
    // at most a path a lane instead of a whole item, so they finish together
    // (1.7 % on the 4M-path benchmark call; on the seven contracts of a
    // smoothed bump the same tail measured 5 % slower, so launches of several
    // contracts keep whole items).
    const size_t nc = jobs.size();
    const uint64_t small = 32, tail = nc == 1 ? warps_total * small : 0;
    P.item_idx.assign(2 * nc + 1, 0u);
    uint64_t n_items = 0;
    for (size_t q = 0; q < nc; ++q) {
        const int ci = order[q];
        ContractDev &C = P.cons[ci];
        const uint64_t n = C.n_paths;
        const uint64_t big = q + 1 < nc || n <= tail ? (n + item - 1) / item : (n - tail) / item;
        C.item_paths = (uint32_t)item;
        C.item_big = (uint32_t)big;
        C.item_small = (uint32_t)small;
        C.path_base = jobs[ci].path_base;
        P.item_idx[q] = (uint32_t)n_items;
        P.item_idx[nc + 1 + q] = (uint32_t)ci;
        const uint64_t rest = n > big * item ? n - big * item : 0;
        n_items += big + (rest + small - 1) / small;
    }
    P.item_idx[nc] = (uint32_t)n_items;
    if (n_items >= (1ull << 31)) raise(KX_INVALID_ARGUMENT, "too many work items in one launch");
    P.n_items = n_items;
    P.grid_blocks = (int)std::min<uint64_t>((uint64_t)full, (n_items + 7) / 8 + 1);
    return P;
}

PathArgs path_args(const PathPlan &P, const PathBuffers &B) {
    PathArgs a{};
    a.progs = static_cast<const KxProgram *>(B.progs);
    a.steps = B.steps;
    a.disc = static_cast<const double *>(B.disc);
    a.cons = static_cast<const ContractDev *>(B.cons);
    a.thr = B.thr;
    a.items = nullptr;  // arithmetic items
    a.item_start = static_cast<const uint32_t *>(B.items);
    a.item_order = static_cast<const int32_t *>(B.items) + P.cons.size() + 1;
    a.n_order = (uint32_t)P.cons.size();
    a.n_items = (uint32_t)P.n_items;
    a.slots = P.slots;
    a.surv_base = P.surv_base;
    a.item_counter = B.counters;
    a.err_word = B.counters + 1;
    a.steps_done = reinterpret_cast<unsigned long long *>(B.counters + 2);
    a.pv = B.pv;
    a.pv_stride = P.total;
    a.statics = P.stat ? B.statics : nullptr;
    bool one_seed = !P.cons.empty();
    for (const ContractDev &c : P.cons) one_seed = one_seed && c.seed == P.cons[0].seed;
    if (one_seed) {  // the Philox key schedule of philox4x32_10, once for the launch
        uint32_t k0 = (uint32_t)P.cons[0].seed, k1 = (uint32_t)(P.cons[0].seed >> 32);
        for (int r = 0; r < 10; ++r) {
            a.rk[2 * r] = k0;
            a.rk[2 * r + 1] = k1;
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        a.rk_ok = 1u;
    }
    return a;
}

void upload_plan(const PathPlan &P, const PathBuffers &B, cudaStream_t s) {
    KX_CUDA(cudaMemcpyAsync(B.progs, P.progs.data(), P.progs.size() * sizeof(KxProgram), cudaMemcpyHostToDevice, s));
    KX_CUDA(cudaMemcpyAsync(B.steps, P.steps.data(), P.steps.size(), cudaMemcpyHostToDevice, s));
    KX_CUDA(cudaMemcpyAsync(B.disc, P.disc.data(), P.disc.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    KX_CUDA(cudaMemcpyAsync(B.cons, P.cons.data(), P.cons.size() * sizeof(ContractDev), cudaMemcpyHostToDevice, s));
    KX_CUDA(cudaMemcpyAsync(B.thr, P.thr.data(), P.thr.size(), cudaMemcpyHostToDevice, s));
    KX_CUDA(cudaMemcpyAsync(B.items, P.item_idx.data(), P.item_idx.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    if (P.stat)
        KX_CUDA(cudaMemcpyAsync(B.statics, P.statics.data(), P.statics.size() * sizeof(StaticDev), cudaMemcpyHostToDevice,
                                s));
}

size_t plan_upload_bytes(const PathPlan &P) {
    return P.progs.size() * sizeof(KxProgram) + P.steps.size() + P.disc.size() * sizeof(double) +
           P.cons.size() * sizeof(ContractDev) + P.thr.size() + P.item_idx.size() * sizeof(uint32_t) +
           P.statics.size() * sizeof(StaticDev);
}

static uint64_t run_paths_v(Ctx &c, std::vector<Job> &jobs, const kx_mc_config &cfg, int ns, uint64_t &stride_out,
                            int minb, bool lean, bool pair) {
    PathPlan P = plan_paths(jobs, cfg, ns, minb, lean, 0, lean && use_static(jobs, ns), pair);
    c.last.path_steps += P.path_steps;
    stride_out = P.total;
    if (P.n_items == 0) return P.total;
    // the plan's tables and the zeroed counters in one device region, staged in pinned memory
    // and uploaded by one copy (each table 256-byte aligned)
    const size_t sz[8] = {P.progs.size() * sizeof(KxProgram), P.steps.size(), P.disc.size() * sizeof(double),
                          P.cons.size() * sizeof(ContractDev), P.thr.size(), P.item_idx.size() * sizeof(uint32_t),
                          P.statics.size() * sizeof(StaticDev), 64};
    const void *src[8] = {P.progs.data(), P.steps.data(), P.disc.data(), P.cons.data(), P.thr.data(),
                          P.item_idx.data(), P.statics.data(), nullptr};
    size_t off[8], total = 0;
    for (int q = 0; q < 8; ++q) {
        off[q] = total;
        total += (sz[q] + 255) & ~size_t(255);
    }
    c.plan.ensure(total);
    c.plan_stage.ensure(total + 64);  // + the counters read back after the launch
    unsigned char *stage = c.plan_stage.as<unsigned char>();
    for (int q = 0; q < 8; ++q) {
        if (src[q] && sz[q]) memcpy(stage + off[q], src[q], sz[q]);
        else if (sz[q]) memset(stage + off[q], 0, sz[q]);
    }
    KX_CUDA(cudaMemcpyAsync(c.plan.p, stage, total, cudaMemcpyHostToDevice, c.stream));
    c.pv.ensure(std::max<uint64_t>(1, P.total * ns) * sizeof(double));
    unsigned char *dp = c.plan.as<unsigned char>();
    const PathBuffers B{dp + off[0], dp + off[1], dp + off[2], dp + off[3], dp + off[4], dp + off[5],
                        reinterpret_cast<uint32_t *>(dp + off[7]), c.pv.as<double>(), dp + off[6]};
    c.last.h2d_bytes += total;
    PathArgs a = path_args(P, B);
    if (cfg.rng == KX_RNG_SHARED_DRAWS) {
        DrawStore &ds = c.draws;
        if (!ds.set) raise(KX_INVALID_ARGUMENT, "no shared draws registered");
        for (auto &j : jobs) {
            const uint64_t need = (uint64_t)(j.dev.n_times - 1) * j.model.draws_per_step();
            if (ds.n_paths < j.dev.n_paths || ds.dpp < need)
                raise(KX_INVALID_ARGUMENT, "shared draws too small: need " + std::to_string(j.dev.n_paths) + " paths x " +
                                               std::to_string(need) + " draws");
        }
        a.z64 = ds.is64 ? ds.z64.as<double>() : nullptr;
        a.z32 = ds.is64 ? nullptr : ds.z32.as<float>();
        a.z_dpp = ds.dpp;
    }
    void *args[] = {&a};
    KX_CUDA(cudaEventRecord(c.ev0, c.stream));
    KX_CUDA(cudaLaunchKernel(P.kfn, dim3(P.grid_blocks), dim3(KX_BLOCK), args, P.smem, c.stream));
    KX_CUDA(cudaEventRecord(c.ev1, c.stream));
    c.last.kernel_launches++;
    c.last.grid_blocks = (uint32_t)P.grid_blocks;
    c.last.block_threads = (uint32_t)KX_BLOCK;
    c.last.path_kernel = P.acc ? 4u : P.stat ? 3u : lean ? 2u : 1u;
    uint32_t *hc = reinterpret_cast<uint32_t *>(stage + total);  // pinned: the counters come back by DMA
    KX_CUDA(cudaMemcpyAsync(hc, B.counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    KX_CUDA(cudaStreamSynchronize(c.stream));
    float ms = 0.f;
    KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.last.kernel_ms += ms;
    uint64_t sim = 0;
    memcpy(&sim, &hc[2], sizeof sim);
    c.last.steps_simulated += sim;
    check_err_word(hc[1]);
    return P.total;
}

void check_err_word(uint32_t err) {
    if (err & KX_ERR_LOOKAHEAD)
        raise(KX_UNSUPPORTED, "an average window is read before it closes (look-ahead average)");
    if (err & KX_ERR_MALFORMED) raise(KX_MALFORMED_CONTRACT, "average window inverted or empty at an evaluation date");
}

// Value `progs` on `grid` with the path kernel, all with the same model,
// config and seed (so on the same simulated paths). Per-contract statistics.
std::vector<Stats> batch_paths(Ctx &c, const std::vector<const Program *> &progs, const Model &m,
                               const kx_mc_config &cfg, const std::vector<double> &grid) {
    std::vector<Job> jobs;
    for (auto *p : progs) jobs.push_back(make_job(*p, m, cfg, grid, {}, 0, 0.0));
    uint64_t stride = 0;
    run_paths(c, jobs, cfg, 1, stride);
    std::vector<StatsJob> sj(progs.size());
    for (size_t i = 0; i < progs.size(); ++i) {
        sj[i].begin = jobs[i].dev.pv_off;
        sj[i].n = cfg.n_paths;
    }
    return device_stats(c, c.pv.as<double>(), stride, sj);
}

void begin_call(Ctx &c) {
    memset(&c.last, 0, sizeof c.last);
    c.last.total_ms = -now_ms();
    c.kahan_stats = false;
}
void end_call(Ctx &c) { c.last.total_ms += now_ms(); }

// ---------------------------------------------------------------------------
// calibration kernels: 8 independent dependency chains per thread, enough
// warps per SM to fill the pipe; the result is stored so nothing is elided.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_peak_mufu(float *out, int iters) {
    float a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = 0.5f + 1e-3f * (threadIdx.x + i);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            float x;
            asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(x) : "f"(a[i]));
            asm volatile("lg2.approx.ftz.f32 %0, %1;" : "=f"(a[i]) : "f"(x));
        }
    }
    float t = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) t += a[i];
    if (t == 12345.f) out[threadIdx.x] = t;
}
__global__ void __launch_bounds__(256) k_peak_fma(float *out, int iters) {
    float a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = 1e-3f * (threadIdx.x + i);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = fmaf(a[i], 0.999f, 1e-4f);
    }
    float t = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) t += a[i];
    if (t == 12345.f) out[threadIdx.x] = t;
}
__global__ void __launch_bounds__(256) k_peak_imad(unsigned *out, int iters) {
    unsigned a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 2654435761u + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = __umulhi(a[i], 0xD2511F53u) + a[i];
    }
    unsigned t = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) t ^= a[i];
    if (t == 12345u) out[threadIdx.x] = t;
}
// The bare simulation loop of the path kernels: one Philox4x32-10 block per
// 4 steps, Box-Muller, the log-space GBM update; no contract, no scheduling.
// Its step rate is the ceiling of any FP32 GBM path kernel on this RNG.
__global__ void __launch_bounds__(256) k_peak_path(float *out, int paths_per_thread, int n_steps) {
    float acc = 0.f;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int q = 0; q < paths_per_thread; ++q) {
        const uint32_t path = tid * (uint32_t)paths_per_thread + (uint32_t)q;
        float y = 0.f;
        for (int b = 0; b < n_steps / 4; ++b) {
            const uint4 w = philox4x32_10(make_uint4((uint32_t)b, path, 0u, 0u), 42u, 0u);
            float z[4];
            box_muller(w.x, w.y, z[0], z[1]);
            box_muller(w.z, w.w, z[2], z[3]);
#pragma unroll
            for (int j = 0; j < 4; ++j) y += 1e-4f + 0.013f * z[j];
        }
        acc += y;
    }
    if (acc == 12345.f) out[threadIdx.x] = acc;
}

// Variance reduction (variance_reduction.rs:186-235): the antithetic pair
// estimator 0.5 (b + a) and the control-variate correction t - 1 (c - bs),
// per path, in the reference's operation order.
__global__ void k_vr_pairs(const double *__restrict__ b, const double *__restrict__ a, uint64_t n,
                           double *__restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = 0.5 * (b[i] + a[i]);
}
__global__ void k_vr_control(const double *__restrict__ t, const double *__restrict__ c, double bs, uint64_t n,
                             double *__restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = t[i] - 1.0 * (c[i] - bs);
}

// norm_cdf and black_scholes_call of numerics.rs:22-71: the Abramowitz-Stegun
// 7.1.26 rational approximation of erfc, as the reference evaluates it (its
// value enters the control-variate price).
static double norm_cdf_as(double x) {
    const double z = x / 1.4142135623730951;  // x / sqrt(2)
    const double sign = z < 0.0 ? -1.0 : 1.0;
    const double a = std::fabs(z);
    const double t = 1.0 / (1.0 + 0.3275911 * a);
    const double poly = ((((1.061405429 * t - 1.453152027) * t) + 1.421413741) * t - 0.284496736) * t + 0.254829592;
    const double erf_abs = 1.0 - poly * t * std::exp(-a * a);
    return 0.5 * (1.0 + sign * erf_abs);
}
static double bs_call_as(double s, double k, double t, double r, double sigma) {
    if (t <= 0.0 || sigma <= 0.0) return std::max(s - k * std::exp(-r * t), 0.0);
    const double vst = sigma * std::sqrt(t);
    const double d1 = (std::log(s / k) + (r + 0.5 * sigma * sigma) * t) / vst;
    const double d2 = d1 - vst;
    return s * norm_cdf_as(d1) - k * std::exp(-r * t) * norm_cdf_as(d2);
}

// A job on the mirrored paths: the diffusion coefficient of every step
// negated, so every normal enters with the opposite sign (the GBM update is
// y + fma(c1, z, c0); -c1 * z = c1 * -z exactly).
static void mirror_job(Job &j) {
    for (auto &c1 : j.tab.c1) c1 = -c1;
    j.dev.uc1 = -j.dev.uc1;
    j.dev.uc1f = -j.dev.uc1f;
}

// price_gbm with variance reduction (pricer.rs:108-230): the target (and the
// control call) valued on the same grid and stream, combined per path on the
// device, summarised with the deterministic chunk statistics.
static kx_price_result price_vr(Ctx &c, const Program &p, const Model &m, const kx_mc_config &cfg,
                                const std::vector<double> &grid, int vr) {
    const bool gbm = m.kind == KX_MODEL_GBM;
    const bool anti = (vr & KX_VR_ANTITHETIC) && gbm;  // other simulators have no antithetic paths
    const bool cv = (vr & KX_VR_CONTROL_VARIATE) != 0;
    const double cs0 = gbm ? m.s0 : 100.0, csig = gbm ? m.sigma : 0.2;  // gbm_params().unwrap_or
    const double t_mat = grid.back();
    Program ctrl;
    double bs = 0.0;
    if (cv) {  // when(at(t_mat), scale(max(spot(asset) - s0, 0), one("USD")))
        char buf[96];
        std::string js = "{\"When\":[{\"At\":";
        snprintf(buf, sizeof buf, "%.17g", t_mat);
        js += buf;
        js += "},{\"Scale\":[{\"Max\":[{\"Sub\":[{\"Spot\":";
        std::string a;  // the asset name as a JSON string
        for (char ch : m.asset) {
            if (ch == '"' || ch == '\\') a += '\\';
            a += ch;
        }
        js += "\"" + a + "\"},{\"Const\":";
        snprintf(buf, sizeof buf, "%.17g", cs0);
        js += buf;
        js += "}]},{\"Const\":0.0}]},{\"One\":\"USD\"}]}]}";
        ctrl.json = js;
        ctrl.ast = parse_contract_json(js.c_str());
        ctrl.plan = compile_plan(*ctrl.ast);
        lower(ctrl);
        bs = bs_call_as(cs0, cs0, t_mat, cfg.rate, csig);
    }
    const uint64_t n = anti ? cfg.n_paths / 2 : cfg.n_paths;
    kx_mc_config c2 = cfg;
    c2.n_paths = n;
    std::vector<Job> jobs;
    jobs.push_back(make_job(p, m, c2, grid, {}, 0, 0.0));  // target
    if (anti) {
        jobs.push_back(jobs[0]);
        mirror_job(jobs.back());
    }
    if (cv) {
        jobs.push_back(make_job(ctrl, m, c2, grid, {}, 0, 0.0));
        if (anti) {
            jobs.push_back(jobs.back());
            mirror_job(jobs.back());
        }
    }
    uint64_t stride = 0;
    run_paths(c, jobs, c2, 1, stride);
    std::vector<StatsJob> sj(1);
    sj[0].n = n;
    // jobs: [target] (plain), [target, mirror] (anti), [target, control] (cv),
    // [target, mirror, control, control mirror] (anti and cv)
    const size_t want = 1 + (anti ? 1 : 0) + (cv ? (anti ? 2 : 1) : 0);
    if (jobs.size() != want) raise(KX_CUDA_ERROR, "variance reduction: unexpected job layout");
    if ((!anti && !cv) || (n == 0 && !(anti && cv)))  // plain paths (no antithetic paths for this model)
        return finish(device_stats(c, c.pv.as<double>(), stride, sj)[0]);
    const double *pv = c.pv.as<double>();
    const int blocks = c.sm_count * 4;
    auto pairs = [&](size_t jb, size_t ja, double *out) {
        k_vr_pairs<<<blocks, 256, 0, c.stream>>>(pv + jobs[jb].dev.pv_off, pv + jobs[ja].dev.pv_off, n, out);
        KX_CUDA(cudaGetLastError());
        c.last.kernel_launches++;
    };
    c.vr.ensure(std::max<uint64_t>(1, 2 * n) * sizeof(double));
    double *v0 = c.vr.as<double>(), *v1 = v0 + n;
    if (anti && !cv) {  // price_antithetic_on_paths
        pairs(0, 1, v0);
        return finish(device_stats(c, v0, n, sj)[0]);
    }
    if (!anti && cv) {  // cv only: price_control_variate_on_paths
        k_vr_control<<<blocks, 256, 0, c.stream>>>(pv + jobs[0].dev.pv_off, pv + jobs[1].dev.pv_off, bs, n, v0);
        KX_CUDA(cudaGetLastError());
        c.last.kernel_launches++;
        return finish(device_stats(c, v0, n, sj)[0]);
    }
    // antithetic + control variate: price_antithetic_with_cv (pricer.rs:185-219); with no pair the
    // reference's formula gives the Black-Scholes value and a 0 / 0 standard error
    if (n) {
        pairs(0, 1, v0);
        pairs(2, 3, v1);
    }
    std::vector<StatsJob> two(2);
    two[0].begin = 0;
    two[0].n = n;
    two[1].begin = n;
    two[1].n = n;
    const std::vector<Stats> st = device_stats(c, v0, 2 * n, two);
    const kx_price_result target = finish(st[0]), control = finish(st[1]);
    kx_price_result r{};
    r.price = target.price - 1.0 * (control.price - bs);
    const uint64_t n_all = 2 * n;
    r.sample_std = target.sample_std;
    r.std_error = target.sample_std / std::sqrt((double)n_all);
    r.ci95_low = r.price - 1.959963984540054 * r.std_error;
    r.ci95_high = r.price + 1.959963984540054 * r.std_error;
    r.n_paths = n_all;
    return r;
}

// The bare Heston loop: Philox4x32-10 + Box-Muller for 2 normals per step and
// the full-truncation Euler step of the path kernels (log spot and variance),
// nothing else: the ceiling of a Heston path kernel on this RNG.
__global__ void __launch_bounds__(256) k_peak_heston(float *out, int paths_per_thread, int n_steps) {
    float acc = 0.f;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const float dt = 1.0f / 252.0f, sq = sqrtf(dt);
    for (int q = 0; q < paths_per_thread; ++q) {
        const uint32_t path = tid * (uint32_t)paths_per_thread + (uint32_t)q;
        float y = 0.f, v = 0.04f;
        for (int b = 0; b < n_steps / 2; ++b) {
            const uint4 w = philox4x32_10(make_uint4((uint32_t)b, path, 0u, 0u), 42u, 0u);
            float z[4];
            box_muller(w.x, w.y, z[0], z[1]);
            box_muller(w.z, w.w, z[2], z[3]);
            heston_step<float>(0.03f, 2.0f, 0.04f, 0.3f, -0.5f, 0.8660254f, KX_HESTON_FULL_TRUNCATION, dt, sq, z[0],
                               z[1], y, v);
            heston_step<float>(0.03f, 2.0f, 0.04f, 0.3f, -0.5f, 0.8660254f, KX_HESTON_FULL_TRUNCATION, dt, sq, z[2],
                               z[3], y, v);
        }
        acc += y + v;
    }
    if (acc == 12345.f) out[threadIdx.x] = acc;
}

}  // namespace kx

using namespace kx;

extern "C" {

kx_status kx_measure_peak(int32_t what, double *ops_per_s) {
    return guarded([&] {
        if (!ops_per_s || what < 0 || what > 4) raise(KX_INVALID_ARGUMENT, "bad arguments");
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        c.misc.ensure(4096);
        const int blocks = c.sm_count * 8, threads = 256, iters = 4096;
        double best = 0.0;
        for (int rep = 0; rep < 4; ++rep) {
            KX_CUDA(cudaEventRecord(c.ev0, c.stream));
            if (what == 0) k_peak_mufu<<<blocks, threads, 0, c.stream>>>(c.misc.as<float>(), iters);
            else if (what == 1) k_peak_fma<<<blocks, threads, 0, c.stream>>>(c.misc.as<float>(), iters);
            else if (what == 2) k_peak_imad<<<blocks, threads, 0, c.stream>>>(c.misc.as<unsigned>(), iters);
            else if (what == 3) k_peak_path<<<blocks, threads, 0, c.stream>>>(c.misc.as<float>(), 4, 256);
            else k_peak_heston<<<blocks, threads, 0, c.stream>>>(c.misc.as<float>(), 4, 256);
            KX_CUDA(cudaGetLastError());
            KX_CUDA(cudaEventRecord(c.ev1, c.stream));
            KX_CUDA(cudaEventSynchronize(c.ev1));
            float ms = 0.f;
            KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
            const double ops = what >= 3 ? (double)blocks * threads * 4 * 256
                                         : (double)blocks * threads * iters * 8 * (what == 0 ? 2 : 1);
            best = std::max(best, ops / (ms * 1e-3));
        }
        *ops_per_s = best;
    });
}


kx_status kx_device_info(char *name, size_t cap, int32_t *sm_count, int32_t *cc_major, int32_t *cc_minor) {
    return guarded([&] {
        Ctx &c = ctx();
        if (name && cap) {
            strncpy(name, c.name.c_str(), cap - 1);
            name[cap - 1] = 0;
        }
        if (sm_count) *sm_count = c.sm_count;
        if (cc_major) *cc_major = c.cc_major;
        if (cc_minor) *cc_minor = c.cc_minor;
    });
}

kx_status kx_last_launch_stats(kx_launch_stats *out) {
    return guarded([&] {
        if (!out) raise(KX_INVALID_ARGUMENT, "out is NULL");
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        *out = c.last;
    });
}

kx_status kx_set_shared_draws(const double *z64, const float *z32, uint64_t n_paths, uint64_t draws_per_path) {
    return guarded([&] {
        if ((z64 == nullptr) == (z32 == nullptr)) raise(KX_INVALID_ARGUMENT, "exactly one of z64 / z32 must be given");
        if (n_paths == 0 || draws_per_path == 0) raise(KX_INVALID_ARGUMENT, "empty draws");
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        DrawStore &d = c.draws;
        const size_t n = (size_t)(n_paths * draws_per_path);
        if (z64) {
            d.z64.ensure(n * sizeof(double));
            KX_CUDA(cudaMemcpy(d.z64.p, z64, n * sizeof(double), cudaMemcpyHostToDevice));
        } else {
            d.z32.ensure(n * sizeof(float));
            KX_CUDA(cudaMemcpy(d.z32.p, z32, n * sizeof(float), cudaMemcpyHostToDevice));
        }
        d.is64 = z64 != nullptr;
        d.n_paths = n_paths;
        d.dpp = draws_per_path;
        d.set = true;
    });
}

kx_status kx_clear_shared_draws(void) {
    return guarded([&] {
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        c.draws.set = false;
    });
}

kx_status kx_price(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg_in, kx_price_result *out,
                   double *per_path_pv) {
    return guarded([&] {
        const Program &p = program_of(prog);
        Model m = model_from_c(model);
        if (!cfg_in) raise(KX_INVALID_ARGUMENT, "config is NULL");
        const int vr = cfg_in->flags & (KX_VR_ANTITHETIC | KX_VR_CONTROL_VARIATE);
        kx_mc_config cfg_v = *cfg_in;
        cfg_v.flags &= ~vr;
        const kx_mc_config *cfg = &cfg_v;
        check_cfg(cfg);
        if (!out) raise(KX_INVALID_ARGUMENT, "out is NULL");
        if (vr && per_path_pv) raise(KX_INVALID_ARGUMENT, "per-path values are not defined with variance reduction");
        validate_model(m);
        auto grid = time_grid_forced(p.plan, cfg->steps_per_year, m.requires_fine_grid());  // pricer.rs:104
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        if (vr) {  // pricer.rs:108-110
            *out = price_vr(c, p, m, *cfg, grid, vr);
            end_call(c);
            return;
        }
        std::vector<Job> jobs;
        jobs.push_back(make_job(p, m, *cfg, grid, {}, 0, 0.0));
        uint64_t stride = cfg->n_paths;
        if (!multi_lean_run(c, jobs[0], *cfg)) run_paths(c, jobs, *cfg, 1, stride);
        std::vector<StatsJob> sj(1);
        sj[0].begin = 0;
        sj[0].n = cfg->n_paths;
        c.kahan_stats = cfg->precision == KX_PREC_FP32_KAHAN;
        *out = finish(device_stats(c, c.pv.as<double>(), stride, sj)[0]);
        if (per_path_pv && cfg->n_paths) {
            KX_CUDA(cudaMemcpyAsync(per_path_pv, c.pv.p, cfg->n_paths * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            KX_CUDA(cudaStreamSynchronize(c.stream));
            c.last.d2h_bytes += cfg->n_paths * sizeof(double);
        }
        end_call(c);
    });
}

kx_status kx_price_chunks(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg, uint64_t first_path,
                          kx_chunk_stats *out, size_t cap, size_t *n_out) {
    return guarded([&] {
        const Program &p = program_of(prog);
        Model m = model_from_c(model);
        check_cfg(cfg);
        if (!out || !n_out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        if (cfg->rng != KX_RNG_PHILOX) raise(KX_INVALID_ARGUMENT, "path ranges draw from Philox");
        if (first_path % KX_STATS_CHUNK != 0) raise(KX_INVALID_ARGUMENT, "first_path must be a multiple of KX_STATS_CHUNK");
        if (first_path + cfg->n_paths > (1ull << 32)) raise(KX_INVALID_ARGUMENT, "first_path + n_paths must be at most 2^32");
        const size_t nc = (size_t)((cfg->n_paths + KX_STATS_CHUNK - 1) / KX_STATS_CHUNK);
        if (cap < nc) raise(KX_INVALID_ARGUMENT, "out holds " + std::to_string(cap) + " chunks, " + std::to_string(nc) +
                                                     " needed");
        validate_model(m);
        auto grid = time_grid_forced(p.plan, cfg->steps_per_year, m.requires_fine_grid());  // pricer.rs:104
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        std::vector<Job> jobs;
        jobs.push_back(make_job(p, m, *cfg, grid, {}, 0, 0.0));
        jobs[0].path_base = (uint32_t)first_path;
        uint64_t stride = 0;
        run_paths(c, jobs, *cfg, 1, stride);
        // the chunks of kx_price's reduction, returned unmerged
        const uint32_t CH = KX_STATS_CHUNK;
        std::vector<ChunkDesc> chunks;
        for (uint64_t b = 0; b < cfg->n_paths; b += CH)
            chunks.push_back(ChunkDesc{b, (uint32_t)std::min<uint64_t>(CH, cfg->n_paths - b), 0});
        if (!chunks.empty()) {
            c.chunks.ensure(chunks.size() * sizeof(ChunkDesc));
            c.chunk_out.ensure(chunks.size() * sizeof(ChunkOut));
            KX_CUDA(cudaMemcpyAsync(c.chunks.p, chunks.data(), chunks.size() * sizeof(ChunkDesc), cudaMemcpyHostToDevice,
                                    c.stream));
            launch_chunk_stats(c.stream, c.pv.as<double>(), c.chunks.as<ChunkDesc>(), c.chunk_out.as<ChunkOut>(),
                               (unsigned)chunks.size());
            c.last.kernel_launches++;
            std::vector<ChunkOut> h(chunks.size());
            KX_CUDA(cudaMemcpyAsync(h.data(), c.chunk_out.p, h.size() * sizeof(ChunkOut), cudaMemcpyDeviceToHost,
                                    c.stream));
            KX_CUDA(cudaStreamSynchronize(c.stream));
            for (size_t q = 0; q < h.size(); ++q) out[q] = kx_chunk_stats{h[q].n, h[q].mean, h[q].m2};
        }
        *n_out = chunks.size();
        end_call(c);
    });
}

kx_status kx_chunk_moments(const double *values, const double *subtrahend, uint32_t n, kx_chunk_stats *out) {
    return guarded([&] {
        if (!out || (n && !values)) raise(KX_INVALID_ARGUMENT, "NULL argument");
        if (n > KX_STATS_CHUNK) raise(KX_INVALID_ARGUMENT, "a chunk holds at most KX_STATS_CHUNK values");
        double mean = 0.0, m2 = 0.0;
        chunk_moments_exact_host(values, subtrahend, n, mean, m2);
        *out = kx_chunk_stats{(double)n, mean, m2};
    });
}

kx_status kx_merge_chunks(const kx_chunk_stats *chunks, size_t n, kx_price_result *out) {
    return guarded([&] {
        if (!out || (n && !chunks)) raise(KX_INVALID_ARGUMENT, "NULL argument");
        std::vector<ChunkOut> h(n);
        for (size_t q = 0; q < n; ++q) h[q] = ChunkOut{chunks[q].n, chunks[q].mean, chunks[q].m2};
        *out = finish(merge_chunks(h.data(), n));
    });
}

kx_status kx_price_portfolio(size_t n, const kx_program *const *progs, const kx_model *models,
                             const kx_mc_config *cfgs, kx_price_result *out, kx_sens *sens) {
    return guarded([&] {
        if (n == 0) return;
        if (!progs || !models || !cfgs || !out) raise(KX_INVALID_ARGUMENT, "NULL array");
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        if (sens) {  // prices and pathwise delta / vega / rho in one adjoint launch per group
            for (size_t i = 0; i < n; ++i) check_cfg(&cfgs[i]);
            portfolio_adjoint(c, n, progs, models, cfgs, out, sens);
            end_call(c);
            return;
        }
        // group by (model kind, precision): one persistent launch per group
        std::vector<size_t> idx(n);
        for (size_t i = 0; i < n; ++i) idx[i] = i;
        std::vector<std::vector<size_t>> groups;
        for (int kind = 0; kind < 2; ++kind)
            for (int prec = 0; prec < 2; ++prec) {
                std::vector<size_t> gset;
                for (size_t i = 0; i < n; ++i)
                    if (models[i].kind == kind && cfgs[i].precision == prec) gset.push_back(i);
                if (!gset.empty()) groups.push_back(gset);
            }
        for (auto &gset : groups) {
            std::vector<Job> jobs;
            for (size_t i : gset) {
                check_cfg(&cfgs[i]);
                if (cfgs[i].rng != KX_RNG_PHILOX) raise(KX_UNSUPPORTED, "portfolio pricing uses Philox normals");
                const Program &p = program_of(progs[i]);
                Model m = model_from_c(&models[i]);
                validate_model(m);
                auto grid = time_grid_forced(p.plan, cfgs[i].steps_per_year, m.requires_fine_grid());
                jobs.push_back(make_job(p, m, cfgs[i], grid, {}, 0, 0.0));
            }
            uint64_t stride = 0;
            run_paths(c, jobs, cfgs[gset[0]], 1, stride);
            std::vector<StatsJob> sj(gset.size());
            for (size_t q = 0; q < gset.size(); ++q) {
                sj[q].begin = jobs[q].dev.pv_off;
                sj[q].n = jobs[q].dev.n_paths;
            }
            auto st = device_stats(c, c.pv.as<double>(), stride, sj);
            for (size_t q = 0; q < gset.size(); ++q) out[gset[q]] = finish(st[q]);
        }
        end_call(c);
    });
}

}  // extern "C"

// The seven CRN scenarios of greeks_gbm (greeks.rs:65-97) at spot s0 and
// volatility sigma: base, spot up / down, vol up / down, rate up / down, all
// with drift = rate as Gbm::new(asset, s0, rate, sigma) (greeks.rs:70). The
// bump sizes (relative ones scaled by the bumped parameter) land in h[3].
static std::vector<Scenario> bump_scenarios(double s0, double sigma, double r, const kx_bumps &b, double h[3]) {
    const double hs = b.relative ? b.spot * s0 : b.spot;
    const double hv = b.relative ? b.vol * sigma : b.vol;
    const double hr = b.relative ? b.rate * r : b.rate;
    if (!(hs > 0) || !(hv > 0) || !(hr > 0)) raise(KX_INVALID_ARGUMENT, "bump sizes must be positive");
    if (sigma - hv < 0) raise(KX_MALFORMED_CONTRACT, "GBM sigma must be non-negative (vol bump too large)");
    h[0] = hs;
    h[1] = hv;
    h[2] = hr;
    return {{s0, r, sigma, r},      {s0 + hs, r, sigma, r}, {s0 - hs, r, sigma, r},    {s0, r, sigma + hv, r},
            {s0, r, sigma - hv, r}, {s0, r + hr, sigma, r + hr}, {s0, r - hr, sigma, r - hr}};
}

// Statistics of the five estimators of one bumped job whose seven scenario
// values per path start at `begin`: price, then delta, gamma, vega and rho as
// per-path central differences (greeks.rs:85-89), in the order of kx_greeks.
static void greek_stats(uint64_t begin, uint64_t n, const double h[3], StatsJob out[5]) {
    const double hs = h[0], hv = h[1], hr = h[2];
    for (int q = 0; q < 5; ++q) {
        out[q] = StatsJob{};
        out[q].begin = begin;
        out[q].n = n;
        out[q].ns = KX_MAX_NS;
        std::fill(out[q].w, out[q].w + 8, 0.0);
    }
    out[0].w[0] = 1.0;                                                                        // price
    out[1].w[1] = 1.0 / (2 * hs); out[1].w[2] = -1.0 / (2 * hs);                              // delta
    out[2].w[1] = 1.0 / (hs * hs); out[2].w[0] = -2.0 / (hs * hs); out[2].w[2] = 1.0 / (hs * hs);  // gamma
    out[3].w[3] = 1.0 / (2 * hv); out[3].w[4] = -1.0 / (2 * hv);                              // vega
    out[4].w[5] = 1.0 / (2 * hr); out[4].w[6] = -1.0 / (2 * hr);                              // rho
}

// The seven reprices of greeks_gbm as plain single-scenario jobs, appended in
// scenario order: each prices Gbm::new(asset, s0, rate, sigma) under McConfig
// {rate, ..cfg} (greeks.rs:69-76) like kx_price, on the same seed and
// therefore the same normals. The lean kernels value each job at the speed
// of a plain price; the seven values of a path sit n_paths apart.
static void append_reprices(std::vector<Job> &jobs, const Program &p, const Model &base, const kx_mc_config &cfg,
                            const std::vector<double> &grid, const std::vector<Scenario> &sc, int smooth = 0,
                            double smooth_w = 0.0) {
    for (const Scenario &s : sc) {
        Model m = base;
        m.s0 = s.s0;
        m.mu = s.mu;
        m.sigma = s.sigma;
        kx_mc_config c2 = cfg;
        c2.rate = s.rate;
        jobs.push_back(make_job(p, m, c2, grid, {}, smooth, smooth_w));
    }
}

static void fill_greeks(const Stats *st5, kx_greeks *out) {
    const kx_price_result r0 = finish(st5[0]), r1 = finish(st5[1]), r2 = finish(st5[2]), r3 = finish(st5[3]),
                          r4 = finish(st5[4]);
    out->price = r0.price; out->price_se = r0.std_error;
    out->delta = r1.price; out->delta_se = r1.std_error;
    out->gamma = r2.price; out->gamma_se = r2.std_error;
    out->vega = r3.price; out->vega_se = r3.std_error;
    out->rho = r4.price; out->rho_se = r4.std_error;
}

// Prices of one contract under many models of one kind with one config, as
// the calibration objectives price their quotes (calibration.rs:72-90,
// 103-126): one path launch for every entry whose price can be formed; an
// entry whose job cannot be built (the reference's price_gbm returns an
// error: an unknown asset, an invalid parameter) is reported in ok[] as 0
// and left out of the launch.
static void calib_prices(Ctx &c, const Program &p, const std::vector<Model> &models, const kx_mc_config &cfg,
                         std::vector<double> &price, std::vector<char> &ok) {
    const size_t n = models.size();
    price.assign(n, std::nan(""));
    ok.assign(n, 0);
    if (n == 0) return;
    auto grid = time_grid_forced(p.plan, cfg.steps_per_year, models[0].requires_fine_grid());
    std::vector<Job> jobs;
    std::vector<size_t> idx;
    for (size_t q = 0; q < n; ++q) {
        try {
            jobs.push_back(make_job(p, models[q], cfg, grid, {}, 0, 0.0));
            idx.push_back(q);
        } catch (const Error &) {
        }
    }
    if (jobs.empty()) return;
    uint64_t stride = 0;
    run_paths(c, jobs, cfg, 1, stride);
    std::vector<StatsJob> sj(jobs.size());
    for (size_t q = 0; q < jobs.size(); ++q) {
        sj[q].begin = jobs[q].dev.pv_off;
        sj[q].n = jobs[q].dev.n_paths;
    }
    auto st = device_stats(c, c.pv.as<double>(), stride, sj);
    for (size_t q = 0; q < jobs.size(); ++q) {
        price[idx[q]] = finish(st[q]).price;
        ok[idx[q]] = 1;
    }
}

// ---------------------------------------------------------------------------
// multilevel Monte Carlo (mlmc.rs, simulate_level_pair)
// ---------------------------------------------------------------------------
static std::vector<double> uniform_grid(double t_max, uint64_t n_steps) {  // simulator.rs:181-184
    const uint64_t n = std::max<uint64_t>(n_steps, 1);
    std::vector<double> g(n + 1);
    for (uint64_t k = 0; k <= n; ++k) g[k] = t_max * (double)k / (double)n;
    return g;
}

static uint64_t mix_seed(uint64_t seed, uint64_t index) {  // simulator.rs:431-433
    return seed ^ (index * 0x9E3779B97F4A7C15ull);
}

static uint64_t mlmc_level_cost(uint32_t l) {  // mlmc.rs:266-272
    return l == 0 ? 1 : (1ull << l) + (1ull << (l - 1));
}

// Every step of a level-pair path has the same coefficients, formed as the
// reference forms them from dt = t_max / n (simulator.rs:328-343, 610-616):
// GBM (mu - sigma^2 / 2) dt and sigma sqrt(dt_f) (the coarse path's normal is
// the sum of two fine ones, so its diffusion keeps sqrt(dt_f)); Heston dt and
// sqrt(dt).
static void set_level_steps(Job &j, const Model &m, double dt, double dt_f) {
    double c0, c1;
    if (m.kind == KX_MODEL_GBM) {
        c0 = (m.mu - 0.5 * m.sigma * m.sigma) * dt;
        c1 = m.sigma * std::sqrt(dt_f);
    } else {
        c0 = dt;
        c1 = std::sqrt(dt);
    }
    for (size_t k = 1; k < j.tab.c0.size(); ++k) {
        j.tab.c0[k] = c0;
        j.tab.c1[k] = c1;
    }
    ContractDev &d = j.dev;
    d.uniform = j.tab.c0.size() > 1 ? 1 : 0;
    d.uc0 = c0;
    d.uc1 = c1;
    d.uc0f = (float)c0;
    d.uc1f = (float)c1;
}

struct LevelRun {
    uint32_t level;
    uint64_t n;
};

// Statistics of Y_l = P_l - P_(l-1) (P_(-1) = 0) on n coupled paths per run
// (mlmc.rs:276-305), runs in increasing level order. The fine paths of all
// runs are one launch, the coarse paths (the _PAIR kernels, reading the same
// Philox streams two fine steps per step) another; both per-path value arrays
// are copied side by side so that a run's coarse value sits at a fixed
// distance from its fine one, and one statistics launch forms fine - coarse.
static std::vector<Stats> mlmc_level_stats(Ctx &c, const Program &p, const Model &m, const kx_mc_config &cfg,
                                           double t_max, uint64_t seed, const std::vector<LevelRun> &runs) {
    std::vector<Job> fine, coarse;
    uint64_t n0 = 0;
    for (const LevelRun &r : runs) {
        const uint32_t l = r.level;
        kx_mc_config c2 = cfg;
        c2.n_paths = r.n;
        c2.seed = mix_seed(mix_seed(seed, l), (uint64_t)l + 1);  // mlmc.rs:288, simulator.rs:345
        const uint64_t nf = 1ull << l;
        const double dt_f = t_max / (double)nf;
        Job jf = make_job(p, m, c2, uniform_grid(t_max, nf), {}, 0, 0.0);
        set_level_steps(jf, m, dt_f, dt_f);
        fine.push_back(std::move(jf));
        if (l == 0) {
            n0 = r.n;
            continue;
        }
        const double dt_c = t_max / (double)(nf / 2);
        Job jc = make_job(p, m, c2, uniform_grid(t_max, nf / 2), {}, 0, 0.0);
        set_level_steps(jc, m, dt_c, dt_f);
        coarse.push_back(std::move(jc));
    }
    uint64_t nfine = 0, ncoarse = 0;
    if (!mlmc_pairs_run(c, fine, coarse, cfg, nfine)) {
        run_paths(c, fine, cfg, 1, nfine);
        c.mlmc.ensure(std::max<uint64_t>(1, 2 * nfine) * sizeof(double));
        if (nfine)
            KX_CUDA(cudaMemcpyAsync(c.mlmc.p, c.pv.p, nfine * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
        if (!coarse.empty()) {
            run_paths_v(c, coarse, cfg, 1, ncoarse, 2, use_lean(coarse, 1), true);
            KX_CUDA(cudaMemcpyAsync(c.mlmc.as<double>() + nfine, c.pv.p, ncoarse * sizeof(double),
                                    cudaMemcpyDeviceToDevice, c.stream));
        }
    }
    // run q >= 1 (level >= 1): fine at f_q, coarse at nfine + f_q - n0, i.e. (nfine - n0) further on
    std::vector<StatsJob> sj(runs.size());
    size_t qc = 0;
    for (size_t q = 0; q < runs.size(); ++q) {
        sj[q].begin = fine[q].dev.pv_off;
        sj[q].n = runs[q].n;
        if (runs[q].level > 0) {
            if (coarse[qc].dev.pv_off + n0 != fine[q].dev.pv_off) raise(KX_CUDA_ERROR, "level pair layout");
            ++qc;
            sj[q].ns = 2;
            sj[q].w[0] = 1.0;
            sj[q].w[1] = -1.0;
        }
    }
    return device_stats(c, c.mlmc.as<double>(), nfine - n0, sj);
}

static void check_mlmc_model(const Model &m) {
    if (m.kind != KX_MODEL_GBM && m.kind != KX_MODEL_HESTON)
        raise(KX_UNSUPPORTED, "this model has no level pairs (simulate_level_pair)");
    if (m.kind == KX_MODEL_HESTON && m.scheme != KX_HESTON_REFERENCE_FLOOR)
        raise(KX_UNSUPPORTED, "level pairs follow the reference Heston scheme (floor after the step)");
}

// CorrelatedGbmN::new (multi_asset.rs:62-83): at least two factors, a
// correlation of their size (implied by the struct), no negative volatility;
// its lower Cholesky factor as numerics::cholesky_lower (numerics.rs:158-183),
// diagonal pivots floored at 0 and columns under a zero pivot set to 0.
static Model multi_model(const kx_multi_gbm &mm) {
    const uint32_t n = mm.n_assets;
    if (n < 2) raise(KX_MALFORMED_CONTRACT, "CorrelatedGbmN: at least 2 assets required");
    if (n > KX_MAX_ASSETS) raise(KX_INVALID_ARGUMENT, "more than KX_MAX_ASSETS factors");
    Model m;
    m.kind = KX_MODEL_MULTI_GBM;
    for (uint32_t i = 0; i < n; ++i) {
        if (!mm.names[i]) raise(KX_INVALID_ARGUMENT, "factor name is NULL");
        if (mm.sigma[i] < 0.0) raise(KX_MALFORMED_CONTRACT, "CorrelatedGbmN: every volatility must be >= 0");
        m.assets.push_back(mm.names[i]);
        m.a_s0.push_back(mm.s0[i]);
        m.a_mu.push_back(mm.mu[i]);
        m.a_sigma.push_back(mm.sigma[i]);
    }
    std::vector<double> l(n * n, 0.0);
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j <= i; ++j) {
            double sum = mm.corr[i * n + j];
            for (uint32_t k = 0; k < j; ++k) sum -= l[i * n + k] * l[j * n + k];
            if (i == j) {
                l[i * n + j] = std::sqrt(std::max(sum, 0.0));
            } else {
                const double pivot = l[j * n + j];
                l[i * n + j] = pivot > 0.0 ? sum / pivot : 0.0;
            }
        }
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j <= i; ++j) m.chol.push_back(l[i * n + j]);
    m.asset = m.assets[0];
    m.s0 = m.a_s0[0];
    m.mu = m.a_mu[0];
    m.sigma = m.a_sigma[0];
    return m;
}

// Upper bound of the per-path values one surface launch keeps in HBM (seven
// doubles per path and cell); larger surfaces run as several launches.
static constexpr uint64_t SURFACE_PV_BYTES = 8ull << 30;

extern "C" {

kx_status kx_greeks_bump(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg,
                         const kx_bumps *bumps, kx_greeks *out) {
    return guarded([&] {
        const Program &p = program_of(prog);
        Model m = model_from_c(model);
        check_cfg(cfg);
        if (!out) raise(KX_INVALID_ARGUMENT, "out is NULL");
        if (m.kind != KX_MODEL_GBM) raise(KX_UNSUPPORTED, "bump-and-reprice Greeks need a GBM model (greeks.rs:60)");
        validate_model(m);
        const kx_bumps b = bumps ? *bumps : kx_bumps{1e-2, 1e-2, 1e-4, 0, 0, 0.0};
        const double r = cfg->rate;
        double h[3];
        std::vector<Scenario> sc = bump_scenarios(m.s0, m.sigma, r, b, h);
        auto grid = time_grid_forced(p.plan, cfg->steps_per_year, false);
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        Model mb = m;
        mb.mu = r;
        std::vector<Job> jobs;
        std::vector<StatsJob> sj(5);
        uint64_t stride = 0;
        // the seven reprices as plain jobs of one launch (the smoothed payoff: each job
        // weighs its barriers with the logistic of the stated width instead of knocking)
        const double w = b.smoothing_width;
        append_reprices(jobs, p, mb, *cfg, grid, sc, b.smooth ? 1 : 0, w > 0 ? w : 1.0);
        run_paths(c, jobs, *cfg, 1, stride);
        stride = cfg->n_paths;
        greek_stats(0, cfg->n_paths, h, sj.data());
        auto st = device_stats(c, c.pv.as<double>(), stride, sj);
        fill_greeks(st.data(), out);
        end_call(c);
    });
}

kx_status kx_greek_surface(const kx_program *prog, const char *asset, const double *spots, size_t n_spots,
                           const double *vols, size_t n_vols, const kx_mc_config *cfg, const kx_bumps *bumps,
                           kx_greeks *out) {
    return guarded([&] {
        const Program &p = program_of(prog);
        check_cfg(cfg);
        if (n_spots == 0 || n_vols == 0) raise(KX_INCONSISTENT_PATH, "empty surface grid");  // surface.rs:113-117
        if (!spots || !vols || !out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        const kx_bumps b = bumps ? *bumps : kx_bumps{1e-2, 1e-2, 1e-4, 0, 0, 0.0};
        const double r = cfg->rate;
        const size_t n_cells = n_spots * n_vols;
        // cell (i, j) = spots[i] x vols[j], row-major (surface.rs:120-124); every
        // cell is greeks_gbm on the same seed, so all cells share each path's normals
        std::vector<std::vector<Scenario>> sc(n_cells);
        std::vector<std::array<double, 3>> h(n_cells);
        for (size_t q = 0; q < n_cells; ++q) {
            Model m{};
            m.kind = KX_MODEL_GBM;
            m.s0 = spots[q / n_vols];
            m.mu = r;
            m.sigma = vols[q % n_vols];
            validate_model(m);
            sc[q] = bump_scenarios(m.s0, m.sigma, r, b, h[q].data());
        }
        auto grid = time_grid_forced(p.plan, cfg->steps_per_year, false);
        kx_model cm{};
        cm.kind = KX_MODEL_GBM;
        cm.s0 = spots[0];
        cm.mu = r;
        cm.sigma = vols[0];
        cm.asset = asset;
        const Model base = model_from_c(&cm);
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        const uint64_t per_cell = std::max<uint64_t>(1, cfg->n_paths) * KX_MAX_NS * sizeof(double);
        const size_t cells_per_launch = (size_t)std::max<uint64_t>(1, SURFACE_PV_BYTES / per_cell);
        for (size_t c0 = 0; c0 < n_cells; c0 += cells_per_launch) {
            const size_t c1 = std::min(n_cells, c0 + cells_per_launch);
            std::vector<Job> jobs;
            for (size_t q = c0; q < c1; ++q) append_reprices(jobs, p, base, *cfg, grid, sc[q]);
            uint64_t stride = 0;
            run_paths(c, jobs, *cfg, 1, stride);
            // estimator-major, so that cells with equal bump sizes share a statistics launch
            const size_t nj = c1 - c0;
            std::vector<StatsJob> tmp(5), sj(5 * nj);
            for (size_t q = 0; q < nj; ++q) {
                greek_stats(jobs[KX_MAX_NS * q].dev.pv_off, cfg->n_paths, h[c0 + q].data(), tmp.data());
                for (int e = 0; e < 5; ++e) sj[e * nj + q] = tmp[e];
            }
            auto st = device_stats(c, c.pv.as<double>(), cfg->n_paths, sj);
            for (size_t q = 0; q < nj; ++q) {
                const Stats st5[5] = {st[q], st[nj + q], st[2 * nj + q], st[3 * nj + q], st[4 * nj + q]};
                fill_greeks(st5, &out[c0 + q]);
            }
        }
        end_call(c);
    });
}

kx_status kx_calib_gbm_prices(const kx_program *prog, const char *asset, const double *spots, size_t n_quotes,
                              const double *sigmas, size_t n_sigmas, const kx_mc_config *cfg, double *out) {
    return guarded([&] {
        const Program &p = program_of(prog);
        check_cfg(cfg);
        if (cfg->rng != KX_RNG_PHILOX) raise(KX_UNSUPPORTED, "calibration pricing uses Philox normals");
        if ((n_quotes && !spots) || (n_sigmas && !sigmas) || (n_quotes != 0 && n_sigmas != 0 && !out))
            raise(KX_INVALID_ARGUMENT, "NULL argument");
        // Gbm::new(asset, spot, rate, sigma) per quote and volatility (calibration.rs:83)
        std::vector<Model> models;
        for (size_t k = 0; k < n_sigmas; ++k)
            for (size_t i = 0; i < n_quotes; ++i) {
                kx_model cm{};
                cm.kind = KX_MODEL_GBM;
                cm.s0 = spots[i];
                cm.mu = cfg->rate;
                cm.sigma = sigmas[k];
                cm.asset = asset;
                models.push_back(model_from_c(&cm));
            }
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        std::vector<double> price;
        std::vector<char> ok;
        calib_prices(c, p, models, *cfg, price, ok);
        for (size_t q = 0; q < models.size(); ++q) out[q] = price[q];  // NaN where the price fails (:86)
        end_call(c);
    });
}

kx_status kx_calib_heston_objective(const kx_program *prog, const char *asset, const double *quotes, size_t n_quotes,
                                    const double *params, size_t n_params, const kx_mc_config *cfg, double *obj,
                                    double *prices) {
    return guarded([&] {
        const Program &p = program_of(prog);
        check_cfg(cfg);
        if (cfg->rng != KX_RNG_PHILOX) raise(KX_UNSUPPORTED, "calibration pricing uses Philox normals");
        if ((n_quotes && !quotes) || (n_params && (!params || !obj))) raise(KX_INVALID_ARGUMENT, "NULL argument");
        // HestonSimulator::new(asset, spot, v0, kappa, theta, sigma_v, rho, rate) (calibration.rs:114-115)
        std::vector<Model> models;
        for (size_t k = 0; k < n_params; ++k)
            for (size_t i = 0; i < n_quotes; ++i) {
                kx_model cm{};
                cm.kind = KX_MODEL_HESTON;
                cm.heston_scheme = KX_HESTON_REFERENCE_FLOOR;
                cm.s0 = quotes[2 * i];
                cm.v0 = params[5 * k];
                cm.kappa = params[5 * k + 1];
                cm.theta = params[5 * k + 2];
                cm.sigma_v = params[5 * k + 3];
                cm.rho = params[5 * k + 4];
                cm.r = cfg->rate;
                cm.asset = asset;
                models.push_back(model_from_c(&cm));
            }
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        std::vector<double> price;
        std::vector<char> ok;
        calib_prices(c, p, models, *cfg, price, ok);
        // the squared errors of the quotes that priced, in quote order, over n_quotes (:111-125)
        for (size_t k = 0; k < n_params; ++k) {
            double sum = 0.0;
            for (size_t i = 0; i < n_quotes; ++i) {
                const size_t q = k * n_quotes + i;
                if (!ok[q]) continue;
                const double d = price[q] - quotes[2 * i + 1];
                sum += d * d;
            }
            obj[k] = sum / (double)n_quotes;
            if (prices)
                for (size_t i = 0; i < n_quotes; ++i) prices[k * n_quotes + i] = price[k * n_quotes + i];
        }
        end_call(c);
    });
}

kx_status kx_mlmc_optimal_allocation(const double *variances, const uint64_t *costs, size_t n, double target_var,
                                     uint64_t *out) {
    return guarded([&] {
        if (n && (!variances || !costs || !out)) raise(KX_INVALID_ARGUMENT, "NULL argument");
        if (n == 0) return;
        if (target_var <= 0.0) {  // mlmc.rs:238-240
            for (size_t k = 0; k < n; ++k) out[k] = 0;
            return;
        }
        double sum_sqrt_vc = 0.0;  // mlmc.rs:241-243
        for (size_t k = 0; k < n; ++k) sum_sqrt_vc += std::sqrt(std::max(variances[k], 0.0) * (double)std::max<uint64_t>(costs[k], 1));
        for (size_t k = 0; k < n; ++k) {
            const double v = std::max(variances[k], 0.0);
            const double cst = (double)std::max<uint64_t>(costs[k], 1);
            if (v <= 0.0) {
                out[k] = 1;
                continue;
            }
            const double nk = (sum_sqrt_vc * std::sqrt(v / cst)) / target_var;
            const double up = std::ceil(nk);
            out[k] = std::max<uint64_t>(up >= 1.8446744073709552e19 ? UINT64_MAX : (uint64_t)up, 1);
        }
    });
}

kx_status kx_mlmc_level_variance(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg,
                                 uint32_t level, uint64_t n_pilot, double *variance) {
    return guarded([&] {
        const Program &p = program_of(prog);
        Model m = model_from_c(model);
        check_cfg(cfg);
        check_mlmc_model(m);
        validate_model(m);
        if (!variance) raise(KX_INVALID_ARGUMENT, "variance is NULL");
        if (level > KX_MLMC_MAX_LEVELS) raise(KX_INVALID_ARGUMENT, "level above KX_MLMC_MAX_LEVELS");
        if (cfg->rng != KX_RNG_PHILOX) raise(KX_UNSUPPORTED, "level pairs draw from Philox");
        if (n_pilot >= (1ull << 32)) raise(KX_INVALID_ARGUMENT, "n_pilot must be below 2^32");
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        *variance = 0.0;
        if (n_pilot) {
            auto st = mlmc_level_stats(c, p, m, *cfg, p.plan.horizon, cfg->seed, {{level, n_pilot}});
            *variance = st[0].n > 1 ? st[0].m2 / (st[0].n - 1.0) : 0.0;  // mean_var, mlmc.rs:318-332
        }
        end_call(c);
    });
}

kx_status kx_price_mlmc(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg,
                        const kx_mlmc_cfg *mcfg, kx_mlmc_result *out) {
    return guarded([&] {
        const Program &p = program_of(prog);
        Model m = model_from_c(model);
        check_cfg(cfg);
        check_mlmc_model(m);
        validate_model(m);
        if (!mcfg || !out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        if (cfg->rng != KX_RNG_PHILOX) raise(KX_UNSUPPORTED, "level pairs draw from Philox");
        const uint32_t L = mcfg->n_levels;
        if (L > KX_MLMC_MAX_LEVELS) raise(KX_INVALID_ARGUMENT, "n_levels above KX_MLMC_MAX_LEVELS");
        if (mcfg->pilot_paths >= (1ull << 32)) raise(KX_INVALID_ARGUMENT, "pilot_paths must be below 2^32");
        const double t_max = p.plan.horizon;  // mlmc.rs:309-312
        std::vector<uint64_t> costs(L + 1);
        for (uint32_t l = 0; l <= L; ++l) costs[l] = mlmc_level_cost(l) * std::max<uint32_t>(mcfg->cost_per_step, 1);
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        // pilot: pilot_paths per level, one pair of launches for all levels (mlmc.rs:126-138)
        std::vector<double> sums(L + 1, 0.0), sumsq(L + 1, 0.0), var(L + 1, 0.0);
        std::vector<uint64_t> counts(L + 1, 0);
        auto absorb = [&](uint32_t l, const Stats &st) {  // the running sums of mlmc.rs:133-135 and :150-152
            sums[l] += st.n * st.mean;
            sumsq[l] += st.m2 + st.n * st.mean * st.mean;
            counts[l] += (uint64_t)st.n;
        };
        if (mcfg->pilot_paths) {
            std::vector<LevelRun> runs;
            for (uint32_t l = 0; l <= L; ++l) runs.push_back({l, mcfg->pilot_paths});
            auto st = mlmc_level_stats(c, p, m, *cfg, t_max, cfg->seed, runs);
            for (uint32_t l = 0; l <= L; ++l) {
                var[l] = st[l].n > 1 ? st[l].m2 / (st[l].n - 1.0) : 0.0;
                absorb(l, st[l]);
            }
        }
        // optimal allocation and the extra paths on a second seed (mlmc.rs:140-166)
        std::vector<uint64_t> extra(L + 1, 0);
        if (kx_mlmc_optimal_allocation(var.data(), costs.data(), L + 1, mcfg->target_variance, extra.data()) != KX_OK)
            raise(KX_INVALID_ARGUMENT, "optimal allocation failed");
        std::vector<LevelRun> runs;
        for (uint32_t l = 0; l <= L; ++l)
            if (extra[l] > 0) {
                if (extra[l] >= (1ull << 32)) raise(KX_INVALID_ARGUMENT, "a level needs 2^32 or more paths");
                runs.push_back({l, extra[l]});
            }
        if (!runs.empty()) {
            auto st = mlmc_level_stats(c, p, m, *cfg, t_max, cfg->seed ^ 0xA5A55A5ADEADBEEFull, runs);
            for (size_t q = 0; q < runs.size(); ++q) absorb(runs[q].level, st[q]);
        }
        // level means and variances, the estimator and its standard error (mlmc.rs:168-214)
        memset(out, 0, sizeof *out);
        out->n_levels = L;
        double price = 0.0, var_q = 0.0;
        uint64_t n_total = 0, total_cost = 0;
        for (uint32_t l = 0; l <= L; ++l) {
            const double n = (double)std::max<uint64_t>(counts[l], 1);
            const double mean = sums[l] / n;
            const double v = counts[l] > 1 ? std::max((sumsq[l] - n * mean * mean) / (n - 1.0), 0.0) : 0.0;
            out->level_means[l] = mean;
            out->level_variances[l] = v;
            out->level_costs[l] = costs[l];
            out->level_paths[l] = counts[l];
            price += mean;
            var_q += v / n;
            n_total += counts[l];
            total_cost += counts[l] * costs[l];
        }
        const double se = std::sqrt(std::max(var_q, 0.0));
        const double Z95 = 1.959963984540054;
        out->price.price = price;
        out->price.std_error = se;
        out->price.sample_std = se * std::sqrt((double)std::max<uint64_t>(n_total, 1));
        out->price.ci95_low = price - Z95 * se;
        out->price.ci95_high = price + Z95 * se;
        out->price.n_paths = n_total;
        out->total_cost = total_cost;
        end_call(c);
    });
}

kx_status kx_price_multi(const kx_program *prog, const kx_multi_gbm *model, const kx_mc_config *cfg,
                         kx_price_result *out, double *per_path_pv) {
    return guarded([&] {
        const Program &p = program_of(prog);
        if (!model || !out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        check_cfg(cfg);
        const Model m = multi_model(*model);
        auto grid = time_grid_forced(p.plan, cfg->steps_per_year, false);
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        begin_call(c);
        std::vector<Job> jobs;
        jobs.push_back(make_job(p, m, *cfg, grid, {}, 0, 0.0));
        uint64_t stride = cfg->n_paths;
        if (!multi_lean_run(c, jobs[0], *cfg)) run_paths(c, jobs, *cfg, 1, stride);
        std::vector<StatsJob> sj(1);
        sj[0].n = cfg->n_paths;
        *out = finish(device_stats(c, c.pv.as<double>(), stride, sj)[0]);
        if (per_path_pv && cfg->n_paths) {
            KX_CUDA(cudaMemcpyAsync(per_path_pv, c.pv.p, cfg->n_paths * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            KX_CUDA(cudaStreamSynchronize(c.stream));
            c.last.d2h_bytes += cfg->n_paths * sizeof(double);
        }
        end_call(c);
    });
}

}  // extern "C"
