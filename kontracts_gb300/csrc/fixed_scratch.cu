// fixed_scratch.cu — kx_price_fixed_scratch: kx_price without device allocation.
//
// Some callers must not allocate device memory while they price: a quoting
// loop for which a cudaMalloc (which can synchronise the whole device and can
// fail under memory pressure) is an unbounded stall, a process whose device
// memory is owned by another allocator or capped by a budget, a service that
// reserves everything it will use at start-up. kx_price grows its buffers on
// demand; this entry point instead keeps every device buffer of a call (the
// contract tables, the work queue, the counters, the per-path values and the
// chunk statistics) in one file-scope device array of fixed size, so a call
// allocates no device memory at all (no cudaMalloc, no cudaFree, no library
// routine that allocates).
//
// Limits: n_paths <= KX_FIXED_MAX_PATHS and grid points <= KX_FIXED_MAX_POINTS
// (larger requests fail with KX_INVALID_ARGUMENT before anything runs);
// Philox draws only; the default register budget of the path kernel (no
// tuning runs). The result equals kx_price's for the same arguments.
//
// Set-up: the first call of a process makes the device current and looks up
// the array's address once (cudaGetSymbolAddress); that first call also
// creates the library's stream and events. Make the first call before any
// stream capture or other phase in which set-up work is unwelcome. The
// address is the array's copy on the library's device (device 0 of the
// process, the one device every entry point of this library uses); the
// array exists on every device that loads the library, but only that copy
// is used.
//
// Zeroing: the work-queue counter, the error word and the step counter at
// the start of the array must be zero when the path kernel starts; every call
// clears them itself (cudaMemsetAsync on the array) before its launch.
// Nothing else needs to start at zero: every other byte a call reads it has
// written first.
//
// Overlap: the array is one per process, shared by every call. Two calls in
// flight at once would overwrite each other's tables and per-path values.
// Calls are therefore serialised: each holds the library lock from its first
// upload until its results are back on the host, and returns only then.
#include <algorithm>
#include <cstring>

#include "launch.hpp"
#include "stats.cuh"

namespace kx {

namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

constexpr uint64_t MAX_PATHS = KX_FIXED_MAX_PATHS;
constexpr uint64_t MAX_POINTS = KX_FIXED_MAX_POINTS;
constexpr uint64_t MIN_ITEM = 64;  // smallest work item of a path launch
constexpr uint64_t MAX_ITEMS = (MAX_PATHS + MIN_ITEM - 1) / MIN_ITEM;
constexpr uint64_t MAX_CHUNKS = (MAX_PATHS + KX_STATS_CHUNK - 1) / KX_STATS_CHUNK;

// byte layout of the array
constexpr size_t OFF_COUNT = 0;  // item counter, error word, steps simulated (u64): zeroed per call
constexpr size_t OFF_PROG = align256(OFF_COUNT + 64);
constexpr size_t OFF_CONS = align256(OFF_PROG + sizeof(KxProgram));
constexpr size_t OFF_THR = align256(OFF_CONS + sizeof(ContractDev));
constexpr size_t OFF_STEPS = align256(OFF_THR + sizeof(double) * KX_MAX_NS * KX_MAX_SPOT);
constexpr size_t OFF_DISC = align256(OFF_STEPS + sizeof(StepRec<double>) * MAX_POINTS);
constexpr size_t OFF_ITEMS = align256(OFF_DISC + sizeof(double) * MAX_POINTS);
constexpr size_t OFF_PV = align256(OFF_ITEMS + sizeof(WorkItem) * MAX_ITEMS);
constexpr size_t OFF_CHUNKS = align256(OFF_PV + sizeof(double) * MAX_PATHS);
constexpr size_t SCRATCH_BYTES = align256(OFF_CHUNKS + sizeof(ChunkOut) * MAX_CHUNKS);
static_assert(SCRATCH_BYTES <= (size_t)10 << 20, "fixed scratch above 10 MiB");

}  // namespace

static __device__ __align__(256) unsigned char g_scratch[SCRATCH_BYTES];

// Address of g_scratch, looked up once with the library's device current.
static unsigned char *g_scratch_ptr = nullptr;

static unsigned char *scratch(Ctx &c) {
    if (g_scratch_ptr) return g_scratch_ptr;
    KX_CUDA(cudaSetDevice(c.device));
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        raise(KX_CUDA_ERROR, std::string("fixed scratch: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    }
    g_scratch_ptr = static_cast<unsigned char *>(p);
    return g_scratch_ptr;
}

// The chunk statistics of k_chunk_stats_exact (a cluster of blocks a chunk,
// chunk_moments_exact_cluster), the chunk bounds taken from the cluster index
// instead of a descriptor table.
__global__ void __cluster_dims__(KX_STATS_CLUSTER, 1, 1) __launch_bounds__(KX_STATS_THREADS, 3)
    k_fixed_stats(const double *__restrict__ vals, uint64_t n, ChunkOut *__restrict__ out) {
    __shared__ uint32_t emax[KX_STATS_THREADS / 32 + KX_STATS_CLUSTER];
    __shared__ uint64_t part[4 * (KX_STATS_THREADS / 32 + KX_STATS_CLUSTER)];
    __shared__ double red[32];
    const uint32_t q = blockIdx.x / KX_STATS_CLUSTER;
    const uint64_t begin = (uint64_t)q * KX_STATS_CHUNK;
    const uint32_t count = (uint32_t)std::min<uint64_t>(KX_STATS_CHUNK, n - begin);
    double mean = 0.0, m2 = 0.0;
    const double *v = vals + begin;
    chunk_moments_exact_cluster<KX_STATS_CLUSTER, KX_STATS_THREADS>([&](uint32_t i) { return v[i]; }, count, emax, part,
                                                                     red, mean, m2);
    if (blockIdx.x % KX_STATS_CLUSTER == 0 && threadIdx.x == 0) out[q] = ChunkOut{(double)count, mean, m2};
}

}  // namespace kx

using namespace kx;

extern "C" kx_status kx_price_fixed_scratch(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg,
                                            kx_price_result *out, double *per_path_pv) {
    return guarded([&] {
        const Program &p = program_of(prog);
        Model m = model_from_c(model);
        check_cfg(cfg);
        if (!out) raise(KX_INVALID_ARGUMENT, "out is NULL");
        if (cfg->rng != KX_RNG_PHILOX) raise(KX_INVALID_ARGUMENT, "fixed-scratch pricing draws from Philox only");
        if (cfg->n_paths > MAX_PATHS)
            raise(KX_INVALID_ARGUMENT, "n_paths " + std::to_string(cfg->n_paths) + " exceeds the fixed scratch limit " +
                                           std::to_string(MAX_PATHS));
        validate_model(m);
        auto grid = time_grid_forced(p.plan, cfg->steps_per_year, m.requires_fine_grid());  // pricer.rs:104
        if (grid.size() > MAX_POINTS)
            raise(KX_INVALID_ARGUMENT, "time grid of " + std::to_string(grid.size()) +
                                           " points exceeds the fixed scratch limit " + std::to_string(MAX_POINTS));
        Ctx &c = ctx();
        std::lock_guard<std::mutex> g(c.mu);
        unsigned char *base = scratch(c);
        begin_call(c);
        const bool f64 = cfg->precision == KX_PREC_FP64;
        std::vector<Job> jobs;
        jobs.push_back(make_job(p, m, *cfg, grid, {}, 0, 0.0));
        Job &j = jobs[0];
        const uint64_t n = cfg->n_paths;

        // tables of the one contract, as a path launch lays them out
        ContractDev d = j.dev;
        d.prog = 0;
        d.step_off = 0;
        d.disc_off = 0;
        d.pv_off = 0;
        std::vector<unsigned char> steps;
        if (f64) pack_steps<double>(j.tab, steps);
        else pack_steps<float>(j.tab, steps);
        std::vector<unsigned char> thr;
        if (f64) {
            thr.resize(j.thr.size() * sizeof(double));
            memcpy(thr.data(), j.thr.data(), thr.size());
        } else {
            thr.resize(j.thr.size() * sizeof(float));
            float *t = reinterpret_cast<float *>(thr.data());
            for (size_t q = 0; q < j.thr.size(); ++q) t[q] = (float)j.thr[q];
        }
        const bool lean = use_lean(jobs, 1) && !lean_has_average(jobs);  // this entry runs no static schedules
        int nv = 0;
        const int minb = variants(j.model.kind, f64, 1, lean, nv)[0];
        const void *kfn = select_kernel(j.model.kind, f64, 1, minb, lean);
        if (!kfn) raise(KX_CUDA_ERROR, "missing kernel variant");
        const int block = KX_BLOCK;
        const uint32_t slots = 2u * (uint32_t)j.prog.n_acc;
        const size_t smem = lean ? 0 : (size_t)slots * block * (f64 ? 8 : 4);  // lean kernels keep no state in shared memory
        const int full = persistent_blocks(kfn, block, smem);
        const uint64_t warps_total = (uint64_t)full * (block / 32);
        uint64_t item = n / std::max<uint64_t>(1, warps_total * 8);
        item = std::max<uint64_t>(MIN_ITEM, std::min<uint64_t>(2048, item));
        item = (item + 31) / 32 * 32;
        std::vector<WorkItem> items;
        for (uint64_t b = 0; b < n; b += item) items.push_back(WorkItem{0, 0, b, std::min(item, n - b)});
        c.last.path_steps += n * (uint64_t)(d.n_times > 0 ? d.n_times - 1 : 0);

        KX_CUDA(cudaMemsetAsync(base + OFF_COUNT, 0, 64, c.stream));
        KX_CUDA(cudaMemcpyAsync(base + OFF_PROG, &j.prog, sizeof(KxProgram), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync(base + OFF_CONS, &d, sizeof(ContractDev), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync(base + OFF_THR, thr.data(), thr.size(), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync(base + OFF_STEPS, steps.data(), steps.size(), cudaMemcpyHostToDevice, c.stream));
        KX_CUDA(cudaMemcpyAsync(base + OFF_DISC, j.tab.disc.data(), j.tab.disc.size() * sizeof(double),
                                cudaMemcpyHostToDevice, c.stream));
        if (!items.empty())
            KX_CUDA(cudaMemcpyAsync(base + OFF_ITEMS, items.data(), items.size() * sizeof(WorkItem),
                                    cudaMemcpyHostToDevice, c.stream));
        c.last.h2d_bytes += sizeof(KxProgram) + sizeof(ContractDev) + thr.size() + steps.size() +
                            j.tab.disc.size() * sizeof(double) + items.size() * sizeof(WorkItem);

        uint32_t *counters = reinterpret_cast<uint32_t *>(base + OFF_COUNT);
        double *pv = reinterpret_cast<double *>(base + OFF_PV);
        ChunkOut *chunks = reinterpret_cast<ChunkOut *>(base + OFF_CHUNKS);
        if (!items.empty()) {
            PathArgs a{};
            a.progs = reinterpret_cast<const KxProgram *>(base + OFF_PROG);
            a.steps = base + OFF_STEPS;
            a.disc = reinterpret_cast<const double *>(base + OFF_DISC);
            a.cons = reinterpret_cast<const ContractDev *>(base + OFF_CONS);
            a.thr = base + OFF_THR;
            a.items = reinterpret_cast<const WorkItem *>(base + OFF_ITEMS);
            a.n_items = (uint32_t)items.size();
            a.slots = slots;
            a.surv_base = slots;
            a.item_counter = counters;
            a.err_word = counters + 1;
            a.steps_done = reinterpret_cast<unsigned long long *>(counters + 2);
            a.pv = pv;
            a.pv_stride = n;
            const int grid_blocks = (int)std::min<uint64_t>((uint64_t)full, (items.size() + 7) / 8 + 1);
            void *args[] = {&a};
            KX_CUDA(cudaEventRecord(c.ev0, c.stream));
            KX_CUDA(cudaLaunchKernel(kfn, dim3(grid_blocks), dim3(block), args, smem, c.stream));
            KX_CUDA(cudaEventRecord(c.ev1, c.stream));
            c.last.kernel_launches++;
            c.last.grid_blocks = (uint32_t)grid_blocks;
            c.last.block_threads = (uint32_t)block;
            c.last.path_kernel = lean ? 2u : 1u;
        }
        const uint64_t nc = (n + KX_STATS_CHUNK - 1) / KX_STATS_CHUNK;
        if (nc) {
            k_fixed_stats<<<(unsigned)nc * KX_STATS_CLUSTER, KX_STATS_THREADS, 0, c.stream>>>(pv, n, chunks);
            KX_CUDA(cudaGetLastError());
            c.last.kernel_launches++;
        }
        ChunkOut h[MAX_CHUNKS];
        uint32_t hc[4] = {0, 0, 0, 0};
        if (nc) KX_CUDA(cudaMemcpyAsync(h, chunks, nc * sizeof(ChunkOut), cudaMemcpyDeviceToHost, c.stream));
        KX_CUDA(cudaMemcpyAsync(hc, counters, sizeof hc, cudaMemcpyDeviceToHost, c.stream));
        if (per_path_pv && n) {
            KX_CUDA(cudaMemcpyAsync(per_path_pv, pv, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            c.last.d2h_bytes += n * sizeof(double);
        }
        KX_CUDA(cudaStreamSynchronize(c.stream));
        c.last.d2h_bytes += nc * sizeof(ChunkOut) + sizeof hc;
        if (!items.empty()) {
            float ms = 0.f;
            KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
            c.last.kernel_ms += ms;
        }
        uint64_t sim = 0;
        memcpy(&sim, &hc[2], sizeof sim);
        c.last.steps_simulated += sim;
        const uint32_t err = hc[1];
        if (err & KX_ERR_LOOKAHEAD)
            raise(KX_UNSUPPORTED, "an average window is read before it closes (look-ahead average)");
        if (err & KX_ERR_MALFORMED) raise(KX_MALFORMED_CONTRACT, "average window inverted or empty at an evaluation date");
        *out = finish(merge_chunks(h, nc));  // chunk order, as kx_price
        end_call(c);
    });
}
