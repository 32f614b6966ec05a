// dpx_batch.cpp — many independent I(q) solves (one PDB leaf each, its own
// grid size, qmax and q list) prepared once and replayed as CUDA graphs.
//
// A solve is the reference's per-structure sequence PDBAmplitude::calculateGrid
// (PDBAmplitude.cpp:319-435) -> CalculateSplines (Grid.cpp:1113-1151) ->
// DomainModel::CalculateIntensityVector's MC between layers (Amplitude.cpp:
// 1168-1247, 2746-2822), which the reference runs one structure at a time.
// Here the solves are packed into waves whose grids fit a device-memory
// budget.  Each wave is one CUDA graph:
//   FP32 with the harmonic method (the default): the fills planned at
//   creation, run in fill batches (as many structures as 8 GiB of scratch
//   holds, each its own part of it): four launches per batch over its job
//   table (moments, group sums, contraction, synthesis with the phi-spline
//   derivatives: launch_harmonic_jobs; the radial tables are the plans');
//   FP32 leaves the harmonic method declines: one direct-sum launch over all of
//   them, then their splines; FP64: the direct sum per structure and splines;
//   the MC averages of all the wave's structures in three launches (bracket
//   tables, average, finalize with the q = 0 terms: launch_average_batch),
//   each structure with its own partial sums;
//   one device-to-host copy of the wave's I(q) into pinned memory.
// All inputs (atoms, form-factor tables, item prefixes, bracket tables and the
// shared direction set, sorted once into its angular order) are uploaded once
// at creation; the grids of a wave live in one pool reused by every wave.
#include "dpx_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

using dpx::Geom;
using namespace dpxh;

struct dpx_batch_s {
    dpx_ctx ctx = nullptr;
    int precision = DPX_FP32;
    int n = 0;
    double eps = 0.0;
    std::vector<int> nq;
    std::vector<size_t> res_off;  // into the result arrays (doubles)
    size_t res_total = 0;
    std::vector<int> wave_first;  // solves [wave_first[w], wave_first[w+1])
    size_t pool_bytes = 0;
    int64_t launches = 0;  // kernels per run
    void* arena = nullptr;
    void* pool = nullptr;
    double* partial = nullptr;
    double* d_res = nullptr;
    double* h_res = nullptr;  // pinned
    std::vector<cudaGraph_t> graphs;
    std::vector<cudaGraphExec_t> execs;
    std::vector<dpxh::HarmPlan> plans;  // FP32 solves the harmonic method fills (arena != nullptr)
    void* hscratch = nullptr;           // the scratch of one fill batch (each fill its own part)
    dpx::HarmJob* hjobs = nullptr;      // [harmonic solves] the fill batches' job tables (device)
    struct FillBatch {
        int wave, first, n;             // jobs [first, first + n) of hjobs
        dpx::HarmShape shape;
    };
    std::vector<FillBatch> fbatches;
    dpx::AvgJob* jobs = nullptr;        // [n] the batched averages' solves (device)
    int* dsort = nullptr;               // the shared directions' angular order (eps = 0), sorted once
};

namespace {

void batch_free(dpx_batch b) {
    if (!b) return;
    set_device(b->ctx);
    cudaStreamSynchronize(b->ctx->stream);
    for (cudaGraphExec_t e : b->execs) cudaGraphExecDestroy(e);
    for (cudaGraph_t g : b->graphs) cudaGraphDestroy(g);
    if (b->arena) cudaFree(b->arena);
    if (b->pool) cudaFree(b->pool);
    if (b->partial) cudaFree(b->partial);
    if (b->d_res) cudaFree(b->d_res);
    if (b->h_res) cudaFreeHost(b->h_res);
    for (dpxh::HarmPlan& p : b->plans) dpxh::harmonic_plan_release(p);
    if (b->hscratch) cudaFree(b->hscratch);
    if (b->hjobs) cudaFree(b->hjobs);
    if (b->jobs) cudaFree(b->jobs);
    if (b->dsort) cudaFree(b->dsort);
    cudaStreamSynchronize(b->ctx->stream);
    ctx_release(b->ctx);
    delete b;
}

// Host staging of one byte arena: returns the offset of the copied block.
struct Stage {
    std::vector<char> h;
    size_t put(const void* src, size_t n) {
        const size_t at = al16(h.size());
        h.resize(at + n);
        if (n) std::memcpy(h.data() + at, src, n);
        return at;
    }
};

struct SolvePlan {
    Geom G;
    int grid_size;
    double qmax;
    size_t grid_off;  // in the pool
    LeafTables lt;  // offsets in the arena
    size_t o_model, o_bq, o_bl, o_bo, o_bi;
    bool origin;  // Q[0] == 0
    dpx::AvgPlan plan;  // pointers filled once the arena exists
    size_t part_off;    // its partial sums and bracket tables in the wave's region
};

}  // namespace

extern "C" {

int dpx_batch_create(dpx_ctx ctx, int n, const dpx_solve_desc* solves, int precision, const double* dirs,
                     int64_t n_samples, double eps, int64_t grid_budget_bytes, dpx_batch* out) {
    if (!ctx || n <= 0 || !solves || !dirs || !out) return fail(DPX_ERR_ARG, "NULL or empty argument");
    if (precision != DPX_FP32 && precision != DPX_FP64) return fail(DPX_ERR_ARG, "bad precision");
    if (n_samples <= 0) return fail(DPX_ERR_ARG, "n_samples must be positive");
    *out = nullptr;
    for (int j = 0; j < n; ++j) {
        const dpx_solve_desc& d = solves[j];
        if (int rc = check_pdb(d.pdb)) return rc;
        if (d.grid_size < 2 || (d.grid_size & 1)) return fail(DPX_ERR_ARG, "solve %d: grid_size must be even", j);
        if (int rc = check_leaf_grid(d.pdb, dpx::make_geom(d.grid_size, d.qmax))) return rc;
        if (!(d.qmax > 0)) return fail(DPX_ERR_ARG, "solve %d: qmax must be positive", j);
        if (d.nq <= 0 || !d.Q) return fail(DPX_ERR_ARG, "solve %d: no q values", j);
        for (int k = 1; k < d.nq; ++k)
            if (!(d.Q[k] >= d.Q[k - 1])) return fail(DPX_ERR_ARG, "solve %d: Q must be ascending", j);
        if (d.Q[0] < 0) return fail(DPX_ERR_ARG, "solve %d: negative q", j);
        if (d.Q[d.nq - 1] > d.qmax * (1.0 + 1e-12)) return fail(DPX_ERR_ARG, "solve %d: q beyond qmax", j);
    }
    if (int rc = set_device(ctx)) return rc;
    const bool fp32 = precision == DPX_FP32;
    const int cpt = fp32 ? ctx->fill_cpt : dpx::kFill64Cells, threads = ctx->fill_threads;
    const bool persistent = ctx->fill_persistent;
    const int poly = ctx->fill_poly;
    if (grid_budget_bytes <= 0) {
        size_t fr = 0, tot = 0;
        DPX_CUDA(cudaMemGetInfo(&fr, &tot));
        grid_budget_bytes = (int64_t)(fr / 2);
    }

    auto* b = new dpx_batch_s;
    b->ctx = ctx;
    ctx_retain(ctx);
    b->precision = precision;
    b->n = n;
    b->eps = eps;

    // waves: solves in order, grid bytes of a wave within the budget
    std::vector<SolvePlan> sp(n);
    b->wave_first.push_back(0);
    size_t wave_bytes = 0;
    for (int j = 0; j < n; ++j) {
        SolvePlan& p = sp[j];
        p.grid_size = solves[j].grid_size;
        p.qmax = solves[j].qmax;
        p.G = dpx::make_geom(p.grid_size, p.qmax);
        const size_t gb = al16((size_t)p.G.P * cell_bytes(precision));
        if (wave_bytes > 0 && (int64_t)(wave_bytes + gb) > grid_budget_bytes) {
            b->pool_bytes = std::max(b->pool_bytes, wave_bytes);
            b->wave_first.push_back(j);
            wave_bytes = 0;
        }
        p.grid_off = wave_bytes;
        wave_bytes += gb;
    }
    b->pool_bytes = std::max(b->pool_bytes, wave_bytes);
    b->wave_first.push_back(n);
    const int n_waves = (int)b->wave_first.size() - 1;

    // the harmonic method plans the FP32 solves it takes (host work and
    // synchronizations here, at creation); the graphs then only replay kernels
    b->plans.resize(n);
    size_t hmax = 0;
    if (fp32 && ctx->fill_method == DPX_FILL_HARMONIC)
        for (int j = 0; j < n; ++j) {
            const int rc = harmonic_plan(ctx->stream, solves[j].pdb, sp[j].G, b->plans[j]);
            if (rc < 0) {
                batch_free(b);
                return rc;
            }
            if (rc == DPX_OK) hmax = std::max(hmax, b->plans[j].scratch_bytes);
        }
    auto harmonic = [&](int j) { return b->plans[j].arena != nullptr; };
    // fill batches: a wave's harmonic fills in order, each batch's scratch (the
    // sum of its fills') within 8 GiB or the largest single fill's
    const size_t fb_budget = std::max(hmax, (size_t)8 << 30);
    size_t hscratch = 0;
    std::vector<size_t> sc_off(n, 0);
    std::vector<int> hjob_of(n, -1);
    int n_hjobs = 0;
    for (int w = 0; w < n_waves; ++w) {
        size_t used = 0;
        for (int j = b->wave_first[w]; j < b->wave_first[w + 1]; ++j) {
            if (!harmonic(j)) continue;
            const size_t need = (b->plans[j].scratch_bytes + 255) & ~size_t(255);
            if (b->fbatches.empty() || b->fbatches.back().wave != w || used + need > fb_budget) {
                b->fbatches.push_back({w, n_hjobs, 0, {}});
                used = 0;
            }
            sc_off[j] = used;
            used += need;
            hscratch = std::max(hscratch, used);
            hjob_of[j] = n_hjobs++;
            b->fbatches.back().n++;
        }
    }

    // staging of every input table
    Stage st;
    size_t partial_max = 0, wave_part = 0;
    int wave = 0;
    for (int j = 0; j < n; ++j) {
        const dpx_solve_desc& d = solves[j];
        const dpx_pdb_desc& pd = d.pdb;
        SolvePlan& p = sp[j];
        const Geom& G = p.G;
        if (!harmonic(j)) stage_leaf(st.h, pd, G, fp32, cpt, p.lt);
        // brackets and the plain identity model
        Brackets B;
        make_brackets(G, p.grid_size, p.qmax, d.nq, d.Q, B);
        p.o_bq = st.put(B.q.data(), B.q.size() * sizeof(double));
        p.o_bl = st.put(B.layer.data(), B.layer.size() * sizeof(int));
        p.o_bo = st.put(B.off.data(), B.off.size() * sizeof(int));
        p.o_bi = st.put(B.qidx.data(), B.qidx.size() * sizeof(int));
        dpx::ModelDev M{};
        M.R[0] = M.R[4] = M.R[8] = 1.0;
        M.sym_scale = 1.0;
        M.plain = 1;
        p.o_model = st.put(&M, sizeof M);  // grid pointer patched below
        dpx::AvgPlan& P = p.plan;
        P = dpx::AvgPlan{};
        P.n_brackets = (int)B.layer.size();
        P.max_q = B.max_q;
        P.n_samples = n_samples;
        P.chunk = eps > 0.0 ? 100 : 128;
        P.chunk_off = eps > 0.0 ? 99 : 0;
        P.n_chunks = (n_samples + P.chunk_off + P.chunk - 1) / P.chunk;
        P.dir_stride = 0;
        P.need_dir = 0;
        P.one_leaf = 1;
        // the solves of a wave average in one launch: each its own partial sums
        if (j == b->wave_first[wave + 1]) {
            ++wave;
            wave_part = 0;
        }
        p.part_off = wave_part;
        wave_part += (((size_t)P.n_brackets * P.n_chunks + (size_t)P.n_brackets * 5) * P.max_q * sizeof(double) +
                      64 + 255) & ~size_t(255);
        partial_max = std::max(partial_max, wave_part);
        p.origin = d.Q[0] == 0.0;
        b->nq.push_back(d.nq);
        b->res_off.push_back(b->res_total);
        b->res_total += (size_t)d.nq;
    }
    const size_t o_dirs = st.put(dirs, (size_t)n_samples * 2 * sizeof(double));
    // per-wave FP32 job tables and tile counters
    std::vector<size_t> o_jobs(n_waves, 0), o_counter(n_waves, 0);
    std::vector<int64_t> wave_tiles(n_waves, 0);
    const size_t jobs_base = al16(st.h.size());
    {
        size_t o = jobs_base;
        for (int w = 0; w < n_waves; ++w) {
            o_jobs[w] = o;
            o = al16(o + (size_t)(b->wave_first[w + 1] - b->wave_first[w]) * sizeof(dpx::FillJob));
            o_counter[w] = o;
            o = al16(o + 64);
        }
        st.h.resize(o, 0);
    }

    // device allocations
    int rc = DPX_OK;
    cudaError_t e = cudaMalloc(&b->arena, st.h.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->pool, b->pool_bytes);
    // with eps = 0 the averages take the shared directions in angular order,
    // sorted once here
    const size_t sort_bytes = eps == 0.0 ? dpx::dir_sort_bytes(n_samples) : 0;
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->partial, partial_max);
    if (e == cudaSuccess && sort_bytes) e = cudaMalloc((void**)&b->dsort, sort_bytes);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->jobs, (size_t)n * sizeof(dpx::AvgJob));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_res, b->res_total * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_res, b->res_total * sizeof(double));
    if (e == cudaSuccess && hscratch) e = cudaMalloc(&b->hscratch, hscratch);
    if (e == cudaSuccess && n_hjobs) e = cudaMalloc((void**)&b->hjobs, (size_t)n_hjobs * sizeof(dpx::HarmJob));
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "batch allocation");
        batch_free(b);
        return rc;
    }
    char* A = static_cast<char*>(b->arena);
    char* pool = static_cast<char*>(b->pool);

    // patch device pointers into the staged models and job tables
    for (int w = 0; w < n_waves; ++w) {
        int64_t tiles = 0;
        std::vector<dpx::FillJob> jobs;
        for (int j = b->wave_first[w]; j < b->wave_first[w + 1]; ++j) {
            SolvePlan& p = sp[j];
            dpx::ModelDev* M = reinterpret_cast<dpx::ModelDev*>(st.h.data() + p.o_model);
            M->grid = pool + p.grid_off;
            if (fp32 && !harmonic(j)) {
                jobs.push_back(make_job(solves[j].pdb, p.lt, A, p.G, pool + p.grid_off, tiles));
                tiles += (p.lt.items + threads - 1) / threads;
            }
            dpx::AvgPlan& P = p.plan;
            P.br_q = reinterpret_cast<const double*>(A + p.o_bq);
            P.br_layer = reinterpret_cast<const int*>(A + p.o_bl);
            P.br_q_off = reinterpret_cast<const int*>(A + p.o_bo);
            P.br_qidx = reinterpret_cast<const int*>(A + p.o_bi);
            P.dirs = reinterpret_cast<const double*>(A + o_dirs);
            P.partial = reinterpret_cast<double*>(reinterpret_cast<char*>(b->partial) + p.part_off);
        }
        if (!jobs.empty()) std::memcpy(st.h.data() + o_jobs[w], jobs.data(), jobs.size() * sizeof(dpx::FillJob));
        wave_tiles[w] = tiles;
    }
    cudaStream_t s = ctx->stream;
    e = cudaMemcpyAsync(b->arena, st.h.data(), st.h.size(), cudaMemcpyHostToDevice, s);
    const int* order = nullptr;
    if (e == cudaSuccess && b->dsort) {
        order = dpx::launch_dir_order(s, reinterpret_cast<const double*>(A + o_dirs), n_samples, b->dsort);
        e = cudaGetLastError();
    }
    // the batched averages' solves
    std::vector<dpx::AvgJob> jobs(n);
    std::vector<int> wave_nbr(n_waves, 0);
    std::vector<int64_t> wave_blocks(n_waves, 0);
    for (int w = 0; w < n_waves; ++w) {
        for (int j = b->wave_first[w]; j < b->wave_first[w + 1]; ++j) {
            dpx::AvgJob& J = jobs[j];
            J = dpx::AvgJob{};
            J.plan = sp[j].plan;
            J.plan.dir_order = order;
            J.model = reinterpret_cast<const dpx::ModelDev*>(A + sp[j].o_model);
            J.res = b->d_res + b->res_off[j];
            J.step = sp[j].G.step;
            J.Lp = sp[j].G.Lp;
            J.origin = sp[j].origin ? 1 : 0;
            wave_nbr[w] = std::max(wave_nbr[w], J.plan.n_brackets);
        }
        wave_blocks[w] = dpx::plan_average_batch(jobs.data() + b->wave_first[w],
                                                 b->wave_first[w + 1] - b->wave_first[w], !fp32);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->jobs, jobs.data(), jobs.size() * sizeof(dpx::AvgJob),
                                              cudaMemcpyHostToDevice, s);
    // the fill batches' job tables: scratch offsets in the batch scratch, grids in the wave's pool
    std::vector<dpx::HarmJob> hjobs(n_hjobs);
    for (int j = 0; j < n; ++j)
        if (hjob_of[j] >= 0) hjobs[hjob_of[j]] = harmonic_job(b->plans[j], sc_off[j], sp[j].grid_off);
    for (auto& fb : b->fbatches) fb.shape = dpx::plan_harmonic_jobs(hjobs.data() + fb.first, fb.n);
    if (e == cudaSuccess && n_hjobs)
        e = cudaMemcpyAsync(b->hjobs, hjobs.data(), hjobs.size() * sizeof(dpx::HarmJob), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "batch upload");
        batch_free(b);
        return rc;
    }

    // record one graph per wave
    for (int w = 0; w < n_waves && !rc; ++w) {
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "cudaStreamBeginCapture");
            break;
        }
        int64_t launches = 0;
        const int j0 = b->wave_first[w], j1 = b->wave_first[w + 1];
        if (fp32) {
            // the wave's harmonic fills: four launches per fill batch
            for (const auto& fb : b->fbatches) {
                if (fb.wave != w || e != cudaSuccess) continue;
                e = dpx::launch_harmonic_jobs(s, b->hjobs + fb.first, fb.n, fb.shape,
                                              static_cast<char*>(b->hscratch), pool, nullptr);
                launches += (fb.shape.moments > 0) + (fb.shape.groups > 0) +
                            (fb.shape.contract > 0) + (fb.shape.synth > 0);
            }
            bool boxes = false;
            int direct = 0;
            for (int j = j0; j < j1; ++j)
                if (!harmonic(j)) {
                    boxes |= sp[j].lt.n_boxes > 0;
                    direct++;
                }
            if (e == cudaSuccess && direct) {
                e = dpx::launch_fill_f32_batch(s, reinterpret_cast<const dpx::FillJob*>(A + o_jobs[w]), direct,
                                               wave_tiles[w], reinterpret_cast<unsigned long long*>(A + o_counter[w]),
                                               cpt, threads, poly, persistent, boxes);
                launches++;
            }
        } else {
            for (int j = j0; j < j1 && e == cudaSuccess; ++j) {
                const SolvePlan& p = sp[j];
                e = launch_leaf_f64(s, solves[j].pdb, p.lt, A, p.G, pool + p.grid_off);
                launches++;
            }
        }
        for (int j = j0; j < j1 && e == cudaSuccess; ++j) {
            const SolvePlan& p = sp[j];
            void* grid = pool + p.grid_off;
            if (!harmonic(j)) {  // the harmonic synthesis writes the derivatives itself
                e = fp32 ? dpx::launch_splines_f32(s, p.G, reinterpret_cast<float4*>(grid))
                         : dpx::launch_splines_f64(s, p.G, reinterpret_cast<double4_32a*>(grid));
                launches++;
            }
        }
        // the wave's averages: bracket tables, average and finalize (with the
        // q = 0 terms), each one launch over all its solves
        const size_t r0 = b->res_off[j0], r1 = (j1 < n) ? b->res_off[j1] : b->res_total;
        if (e == cudaSuccess) e = cudaMemsetAsync(b->d_res + r0, 0, (r1 - r0) * sizeof(double), s);
        if (e == cudaSuccess)
            e = dpx::launch_average_batch(s, !fp32, b->jobs + j0, j1 - j0, wave_nbr[w], wave_blocks[w], eps);
        launches += 3;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b->h_res + r0, b->d_res + r0, (r1 - r0) * sizeof(double), cudaMemcpyDeviceToHost, s);
        const cudaError_t ec = cudaStreamEndCapture(s, &g);
        if (e == cudaSuccess) e = ec;
        if (e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            rc = cuda_fail(e, "batch graph capture");
            break;
        }
        b->graphs.push_back(g);
        cudaGraphExec_t x = nullptr;
        e = cudaGraphInstantiate(&x, g, 0);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "cudaGraphInstantiate");
            break;
        }
        b->execs.push_back(x);
        b->launches += launches;
    }
    if (rc) {
        batch_free(b);
        return rc;
    }
    *out = b;
    return DPX_OK;
}

int dpx_batch_launch(dpx_batch b) {
    if (!b) return fail(DPX_ERR_ARG, "batch is NULL");
    if (int rc = set_device(b->ctx)) return rc;
    for (cudaGraphExec_t x : b->execs) DPX_CUDA(cudaGraphLaunch(x, b->ctx->stream));
    return DPX_OK;
}

int dpx_batch_run(dpx_batch b) {
    if (int rc = dpx_batch_launch(b)) return rc;
    DPX_CUDA(cudaStreamSynchronize(b->ctx->stream));
    return DPX_OK;
}

int dpx_batch_info(dpx_batch b, int* n_waves, int64_t* kernels_per_run, int64_t* pool_bytes) {
    if (!b) return fail(DPX_ERR_ARG, "batch is NULL");
    if (n_waves) *n_waves = (int)b->execs.size();
    if (kernels_per_run) *kernels_per_run = b->launches;
    if (pool_bytes) *pool_bytes = (int64_t)b->pool_bytes;
    return DPX_OK;
}

int dpx_batch_result(dpx_batch b, int j, double* res) {
    if (!b || !res) return fail(DPX_ERR_ARG, "NULL argument");
    if (j < 0 || j >= b->n) return fail(DPX_ERR_ARG, "solve %d out of range", j);
    std::memcpy(res, b->h_res + b->res_off[j], (size_t)b->nq[j] * sizeof(double));
    return DPX_OK;
}

int dpx_batch_destroy(dpx_batch b) {
    if (!b) return fail(DPX_ERR_ARG, "batch is NULL");
    batch_free(b);
    return DPX_OK;
}

}  // extern "C"
