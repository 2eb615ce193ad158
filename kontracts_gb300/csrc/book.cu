// book.cu — a book of contracts priced by replaying one CUDA graph.
//
// kx_price_portfolio rebuilds and re-uploads every table on each call. A
// book is built once: the contracts are lowered and bound, grouped by (model,
// precision, kernel family), their tables uploaded to device memory the book
// owns, the launch shape of every group tuned on the book itself, and the
// whole pricing step captured in one CUDA graph:
//
//   per group: clear the 3 work counters, one persistent path kernel over the
//   group's (contract, path-block) work queue;
//   one chunk-statistics launch over every contract's per-path values;
//   copy the chunk statistics and counters to pinned host memory.
//
// kx_book_price replays the graph and merges the chunk statistics of each
// contract on the host (the same fixed-order merge as kx_price, so a book
// gives exactly the prices kx_price gives contract by contract).
// kx_book_set_models re-binds the contracts to new model parameters (same
// model kinds) and re-uploads the tables in place, so the same graph prices
// the book under the new market (calibration and risk loops).
//
// Tuning (KX_BOOK_TUNE): each group is timed at every register budget of its
// kernel family and at three work-item sizes (paths per (contract, block)
// item); the fastest is kept. All choices compute every path identically.
#include <algorithm>
#include <cstring>
#include <memory>

#include "launch.hpp"

struct kx_book {
    struct Group {
        std::vector<size_t> members;  // contract indices
        kx_mc_config cfg;
        kx::PathPlan plan;
        kx::PathBuffers B;
        size_t pv_base = 0;  // first per-path value of the group in the value arena
        float tuned_ms = 0.f;
        int family = 0;      // 0 k_paths, 1 k_lean, 2 k_lean with static schedules
    };
    std::vector<Group> groups;
    std::vector<const kx::Program *> progs;
    std::vector<kx::Model> models;
    std::vector<kx_mc_config> cfgs;
    std::vector<std::vector<double>> grids;
    std::vector<uint64_t> chunk_first;  // per contract, into the chunk table (size n + 1)
    size_t n_chunks = 0;
    uint64_t path_steps = 0, n_paths = 0;
    void *arena = nullptr;
    kx::ChunkDesc *d_chunks = nullptr;
    kx::ChunkOut *d_out = nullptr;
    double *d_pv = nullptr;
    uint32_t *d_counters = nullptr;  // 16 u32 per group
    kx::ChunkOut *h_out = nullptr;   // pinned
    uint32_t *h_counters = nullptr;  // pinned, 16 u32 per group
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double tune_ms = 0.0;
};

namespace kx {

namespace {

constexpr size_t A256(size_t x) { return (x + 255) & ~size_t(255); }

std::vector<Job> group_jobs(kx_book &b, const kx_book::Group &g) {
    std::vector<Job> jobs;
    for (size_t i : g.members) jobs.push_back(make_job(*b.progs[i], b.models[i], b.cfgs[i], b.grids[i], {}, 0, 0.0));
    return jobs;
}

// Device pointers of a group's tables inside the arena (the sizes do not
// depend on the launch shape the tuner tries).
struct Region {
    size_t progs, steps, disc, cons, thr, items, statics;
};

Region region_sizes(const PathPlan &P) {
    return Region{A256(P.progs.size() * sizeof(KxProgram)), A256(P.steps.size()), A256(P.disc.size() * sizeof(double)),
                  A256(P.cons.size() * sizeof(ContractDev)), A256(P.thr.size()),
                  A256(P.item_idx.size() * sizeof(uint32_t)), A256(P.statics.size() * sizeof(StaticDev))};
}

float time_group(Ctx &c, kx_book &b, kx_book::Group &g, std::vector<Job> &jobs, int minb, uint64_t item) {
    PathPlan P = plan_paths(jobs, g.cfg, 1, minb, g.plan.lean, item, g.plan.stat);
    upload_plan(P, g.B, c.stream);
    KX_CUDA(cudaMemsetAsync(g.B.counters, 0, 64, c.stream));
    PathArgs a = path_args(P, g.B);
    void *args[] = {&a};
    KX_CUDA(cudaEventRecord(c.ev0, c.stream));
    KX_CUDA(cudaLaunchKernel(P.kfn, dim3(P.grid_blocks), dim3(KX_BLOCK), args, P.smem, c.stream));
    KX_CUDA(cudaEventRecord(c.ev1, c.stream));
    KX_CUDA(cudaEventSynchronize(c.ev1));
    float ms = 0.f;
    KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    (void)b;
    return ms;
}

void capture(Ctx &c, kx_book &b) {
    if (b.exec) {
        cudaGraphExecDestroy(b.exec);
        b.exec = nullptr;
    }
    if (b.graph) {
        cudaGraphDestroy(b.graph);
        b.graph = nullptr;
    }
    KX_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    for (auto &g : b.groups) {
        if (g.plan.n_items == 0) continue;
        if (err == cudaSuccess) err = cudaMemsetAsync(g.B.counters, 0, 64, c.stream);
        PathArgs a = path_args(g.plan, g.B);
        void *args[] = {&a};
        if (err == cudaSuccess)
            err = cudaLaunchKernel(g.plan.kfn, dim3(g.plan.grid_blocks), dim3(KX_BLOCK), args, g.plan.smem, c.stream);
    }
    if (err == cudaSuccess && b.n_chunks) {
        // one launch over every contract's chunks (unit weight, one scenario)
        launch_chunk_stats(c.stream, b.d_pv, b.d_chunks, b.d_out, (unsigned)b.n_chunks);
        err = cudaMemcpyAsync(b.h_out, b.d_out, b.n_chunks * sizeof(ChunkOut), cudaMemcpyDeviceToHost, c.stream);
    }
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(b.h_counters, b.d_counters, b.groups.size() * 64, cudaMemcpyDeviceToHost, c.stream);
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(c.stream, &graph);
    if (err != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cuda_check(err != cudaSuccess ? err : e2, "capture of the book graph");
    }
    b.graph = graph;
    KX_CUDA(cudaGraphInstantiate(&b.exec, b.graph, 0));
}

void free_book(kx_book *b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->arena) cudaFree(b->arena);
    if (b->h_out) cudaFreeHost(b->h_out);
    if (b->h_counters) cudaFreeHost(b->h_counters);
    delete b;
}

}  // namespace

}  // namespace kx

using namespace kx;

extern "C" {

kx_status kx_book_create(size_t n, const kx_program *const *progs, const kx_model *models, const kx_mc_config *cfgs,
                         uint32_t flags, kx_book **out) {
    return guarded([&] {
        if (!out) raise(KX_INVALID_ARGUMENT, "out is NULL");
        *out = nullptr;
        if (n == 0) raise(KX_INVALID_ARGUMENT, "empty book");
        if (!progs || !models || !cfgs) raise(KX_INVALID_ARGUMENT, "NULL array");
        if (flags & ~KX_BOOK_TUNE) raise(KX_INVALID_ARGUMENT, "unknown book flags");
        std::unique_ptr<kx_book, void (*)(kx_book *)> b(new kx_book(), free_book);
        for (size_t i = 0; i < n; ++i) {
            check_cfg(&cfgs[i]);
            if (cfgs[i].rng != KX_RNG_PHILOX) raise(KX_UNSUPPORTED, "a book draws from Philox");
            const Program &p = program_of(progs[i]);
            Model m = model_from_c(&models[i]);
            validate_model(m);
            b->progs.push_back(&p);
            b->models.push_back(m);
            b->cfgs.push_back(cfgs[i]);
            b->grids.push_back(time_grid_forced(p.plan, cfgs[i].steps_per_year, m.requires_fine_grid()));
        }
        Ctx &c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        begin_call(c);
        // groups: (model kind, precision, kernel family: 3 static with a running average,
        // 2 static, 1 lean with the general handler, 0 k_paths)
        std::vector<int> fam(n);
        for (size_t i = 0; i < n; ++i) {
            std::vector<Job> one;
            one.push_back(make_job(*b->progs[i], b->models[i], b->cfgs[i], b->grids[i], {}, 0, 0.0));
            fam[i] = use_static(one, 1) ? (lean_has_average(one) ? 3 : 2) : use_lean(one, 1) ? 1 : 0;
        }
        for (int kind = 0; kind < 2; ++kind)
            for (int prec = 0; prec < 2; ++prec)
                for (int f = 3; f >= 0; --f) {
                    kx_book::Group g;
                    for (size_t i = 0; i < n; ++i)
                        if (b->models[i].kind == kind && b->cfgs[i].precision == prec && fam[i] == f) g.members.push_back(i);
                    if (g.members.empty()) continue;
                    g.cfg = b->cfgs[g.members[0]];
                    g.family = f;
                    b->groups.push_back(std::move(g));
                }
        // plans at the default shape; arena sized for the largest item table
        size_t bytes = 0;
        std::vector<Region> regs;
        std::vector<std::vector<Job>> jobs(b->groups.size());
        for (size_t q = 0; q < b->groups.size(); ++q) {
            auto &g = b->groups[q];
            jobs[q] = group_jobs(*b, g);
            int nv = 0;
            const bool lean = g.family >= 1;
            const int *vs = variants(b->models[g.members[0]].kind, g.cfg.precision == KX_PREC_FP64, 1, lean, nv);
            g.plan = plan_paths(jobs[q], g.cfg, 1, vs[0], lean, 0, g.family >= 2);
            regs.push_back(region_sizes(g.plan));
            const Region &r = regs.back();
            bytes += r.progs + r.steps + r.disc + r.cons + r.thr + r.items + r.statics;
            g.pv_base = b->n_paths;
            b->n_paths += g.plan.total;
            b->path_steps += g.plan.path_steps;
        }
        // chunk table: every contract's per-path values in fixed chunks
        std::vector<ChunkDesc> chunks;
        b->chunk_first.assign(n + 1, 0);
        std::vector<std::vector<ChunkDesc>> per(n);
        for (size_t q = 0; q < b->groups.size(); ++q) {
            auto &g = b->groups[q];
            for (size_t k = 0; k < g.members.size(); ++k) {
                const uint64_t begin = g.pv_base + jobs[q][k].dev.pv_off, np = jobs[q][k].dev.n_paths;
                for (uint64_t o = 0; o < np; o += KX_STATS_CHUNK)
                    per[g.members[k]].push_back(
                        ChunkDesc{begin + o, (uint32_t)std::min<uint64_t>(KX_STATS_CHUNK, np - o), 0});
            }
        }
        for (size_t i = 0; i < n; ++i) {
            b->chunk_first[i] = chunks.size();
            chunks.insert(chunks.end(), per[i].begin(), per[i].end());
        }
        b->chunk_first[n] = chunks.size();
        b->n_chunks = chunks.size();
        const size_t off_pv = A256(bytes);
        const size_t off_cnt = A256(off_pv + std::max<uint64_t>(1, b->n_paths) * sizeof(double));
        const size_t off_ch = A256(off_cnt + b->groups.size() * 64);
        const size_t off_out = A256(off_ch + std::max<size_t>(1, b->n_chunks) * sizeof(ChunkDesc));
        const size_t total = A256(off_out + std::max<size_t>(1, b->n_chunks) * sizeof(ChunkOut));
        KX_CUDA(cudaMalloc(&b->arena, total));
        KX_CUDA(cudaMallocHost((void **)&b->h_out, std::max<size_t>(1, b->n_chunks) * sizeof(ChunkOut)));
        KX_CUDA(cudaMallocHost((void **)&b->h_counters, b->groups.size() * 64));
        unsigned char *base = static_cast<unsigned char *>(b->arena);
        b->d_pv = reinterpret_cast<double *>(base + off_pv);
        b->d_counters = reinterpret_cast<uint32_t *>(base + off_cnt);
        b->d_chunks = reinterpret_cast<ChunkDesc *>(base + off_ch);
        b->d_out = reinterpret_cast<ChunkOut *>(base + off_out);
        size_t o = 0;
        for (size_t q = 0; q < b->groups.size(); ++q) {
            auto &g = b->groups[q];
            const Region &r = regs[q];
            g.B.progs = base + o; o += r.progs;
            g.B.steps = base + o; o += r.steps;
            g.B.disc = base + o; o += r.disc;
            g.B.cons = base + o; o += r.cons;
            g.B.thr = base + o; o += r.thr;
            g.B.items = base + o; o += r.items;
            g.B.statics = base + o; o += r.statics;
            g.B.counters = b->d_counters + 16 * q;
            g.B.pv = b->d_pv + g.pv_base;
        }
        if (b->n_chunks)
            KX_CUDA(cudaMemcpyAsync(b->d_chunks, chunks.data(), chunks.size() * sizeof(ChunkDesc),
                                    cudaMemcpyHostToDevice, c.stream));
        // tuning: register budget x work-item size, timed on the book itself
        const double t0 = now_ms();
        for (size_t q = 0; q < b->groups.size(); ++q) {
            auto &g = b->groups[q];
            if (g.plan.n_items == 0) continue;
            int minb = g.plan.minb;
            uint64_t item = g.plan.item_paths;
            if (flags & KX_BOOK_TUNE) {
                int nv = 0;
                const int *vs = variants(g.plan.model, g.plan.f64, 1, g.plan.lean, nv);
                const uint64_t items[3] = {256, 1024, g.plan.item_paths};
                float best = 1e30f;
                time_group(c, *b, g, jobs[q], vs[0], item);  // warm-up
                for (int v = 0; v < nv; ++v)
                    for (uint64_t it : items) {
                        const float ms = time_group(c, *b, g, jobs[q], vs[v], it);
                        if (ms < best) { best = ms; minb = vs[v]; item = it; }
                    }
                g.tuned_ms = best;
            }
            g.plan = plan_paths(jobs[q], g.cfg, 1, minb, g.plan.lean, item, g.plan.stat);
            upload_plan(g.plan, g.B, c.stream);
            c.last.h2d_bytes += plan_upload_bytes(g.plan);
        }
        b->tune_ms = now_ms() - t0;
        KX_CUDA(cudaStreamSynchronize(c.stream));
        capture(c, *b);
        end_call(c);
        *out = b.release();
    });
}

kx_status kx_book_price(kx_book *b, kx_price_result *out) {
    return guarded([&] {
        if (!b || !out) raise(KX_INVALID_ARGUMENT, "NULL argument");
        Ctx &c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        begin_call(c);
        KX_CUDA(cudaEventRecord(c.ev0, c.stream));
        KX_CUDA(cudaGraphLaunch(b->exec, c.stream));
        KX_CUDA(cudaEventRecord(c.ev1, c.stream));
        KX_CUDA(cudaStreamSynchronize(c.stream));
        float ms = 0.f;
        KX_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        c.last.kernel_ms = ms;
        c.last.path_steps = b->path_steps;
        c.last.d2h_bytes = b->n_chunks * sizeof(ChunkOut) + b->groups.size() * 64;
        for (size_t q = 0; q < b->groups.size(); ++q) {
            const uint32_t *hc = b->h_counters + 16 * q;
            uint64_t sim = 0;
            memcpy(&sim, hc + 2, sizeof sim);
            c.last.steps_simulated += sim;
            check_err_word(hc[1]);
            if (b->groups[q].plan.n_items) c.last.kernel_launches++;
            c.last.path_kernel = b->groups[q].plan.acc ? 4u : b->groups[q].plan.stat ? 3u : b->groups[q].plan.lean ? 2u : 1u;
        }
        if (b->n_chunks) c.last.kernel_launches++;
        const size_t n = b->progs.size();
        for (size_t i = 0; i < n; ++i)
            out[i] = finish(merge_chunks(b->h_out + b->chunk_first[i], b->chunk_first[i + 1] - b->chunk_first[i]));
        end_call(c);
    });
}

kx_status kx_book_set_models(kx_book *b, const kx_model *models) {
    return guarded([&] {
        if (!b || !models) raise(KX_INVALID_ARGUMENT, "NULL argument");
        const size_t n = b->progs.size();
        std::vector<Model> ms;
        for (size_t i = 0; i < n; ++i) {
            Model m = model_from_c(&models[i]);
            validate_model(m);
            if (m.kind != b->models[i].kind) raise(KX_INVALID_ARGUMENT, "a book keeps the model kind of each contract");
            ms.push_back(m);
        }
        Ctx &c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        for (size_t i = 0; i < n; ++i) {
            // the grid depends on the model only through requires_fine_grid, fixed by the kind
            b->models[i] = ms[i];
        }
        for (auto &g : b->groups) {
            if (g.plan.n_items == 0) continue;
            std::vector<Job> jobs = group_jobs(*b, g);
            if (use_lean(jobs, 1) != g.plan.lean || (g.plan.stat && !use_static(jobs, 1)))
                raise(KX_INVALID_ARGUMENT, "new model parameters change a contract's kernel family");
            PathPlan P = plan_paths(jobs, g.cfg, 1, g.plan.minb, g.plan.lean, g.plan.item_paths, g.plan.stat);
            if (P.steps.size() != g.plan.steps.size() || P.n_items != g.plan.n_items ||
                P.statics.size() != g.plan.statics.size() ||
                P.grid_blocks != g.plan.grid_blocks || P.smem != g.plan.smem)
                raise(KX_INVALID_ARGUMENT, "new model parameters change the book's layout");
            upload_plan(P, g.B, c.stream);
            g.plan = std::move(P);
        }
        KX_CUDA(cudaStreamSynchronize(c.stream));
    });
}

kx_status kx_book_get_info(const kx_book *b, kx_book_info *info) {
    return guarded([&] {
        if (!b || !info) raise(KX_INVALID_ARGUMENT, "NULL argument");
        memset(info, 0, sizeof *info);
        info->n_contracts = (uint32_t)b->progs.size();
        info->n_groups = (uint32_t)b->groups.size();
        info->n_paths = b->n_paths;
        info->path_steps = b->path_steps;
        info->tune_ms = b->tune_ms;
        for (size_t q = 0; q < b->groups.size() && q < 4; ++q) {
            info->group_kernel[q] = b->groups[q].plan.acc ? 4u : b->groups[q].plan.stat ? 3u : b->groups[q].plan.lean ? 2u : 1u;
            info->group_minb[q] = (uint32_t)b->groups[q].plan.minb;
            info->group_item_paths[q] = (uint32_t)b->groups[q].plan.item_paths;
            info->group_contracts[q] = (uint32_t)b->groups[q].members.size();
        }
    });
}

void kx_book_free(kx_book *b) {
    if (!b) return;
    try {
        Ctx &c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        free_book(b);
    } catch (...) {
    }
}

}  // extern "C"
