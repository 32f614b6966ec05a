// dpx_server.cpp — the serving engine: a continuous-batching request loop for
// I(q) solves on one GPU.
//
// The reference runs one job at a time on a job thread (JobManager.cpp:151-206,
// ERROR_JOBRUNNING while busy) and refills every amplitude grid per job unless
// its own cache file matches.  Here one worker thread owns the device and, on
// every turn of its loop:
//   1. retires requests whose completion event has fired (results copied out,
//      their grids unpinned, their scratch released);
//   2. admits pending requests in arrival order while the device-memory budget
//      allows (grids not yet resident + the request's scratch), evicting
//      unpinned cached grids least-recently-used first; a request that does not
//      fit yet lets later, smaller ones pass;
//   3. fills every grid the newly admitted requests miss in ONE batched FP32
//      fill launch on the fill stream (FP64: one launch per grid), then splines;
//   4. queues each admitted request's orientation average on one of several
//      streams, after the fill events of its grids: requests that arrive while
//      others run overlap with them on the device.
// Grids stay resident after their requests finish, keyed by the leaf's content
// (or a caller key) and the grid parameters, so fitting-style repeats that only
// change placements (R_k, t_k) skip the fill entirely.
#include "dpx_host.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

using dpx::Geom;
using namespace dpxh;

namespace {

using Clock = std::chrono::steady_clock;

uint64_t fnv(uint64_t h, const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

struct LeafCopy {
    std::vector<float> atoms;  // 4 per atom, host
    std::vector<int> api;
    std::vector<double> coeffs, rads;
    int n_ions = 0, flags = 0;
    double sol_ed = 0, c1 = 1, scale = 1;
    bool has_center = false;
    double center[3] = {0, 0, 0};
    std::vector<float> boxes;  // 8 per voxelized-solvent box
    double voxel_step = 0;     // the voxel edge the boxes were built on (the harmonic fill needs it)
    uint64_t key = 0;  // content (or caller) key, before the grid parameters
};

struct GridEntry {
    uint64_t key = 0;
    int grid_size = 0;
    double qmax = 0;
    int precision = DPX_FP32;
    Geom G{};
    void* cells = nullptr;
    size_t bytes = 0;
    int pins = 0;
    uint64_t last_use = 0;
    bool filled = false;  // fill + splines queued
    cudaEvent_t ready = nullptr;
    const LeafCopy* src = nullptr;  // leaf to fill from (valid while its request is admitted)
};

struct Request {
    uint64_t ticket = 0;
    std::vector<LeafCopy> leaves;
    std::vector<int> model_leaf, n_copies;
    std::vector<double> rot, tr, copy_rot, copy_tr, sym_scale;
    int grid_size = 0, precision = DPX_FP32, nq = 0;
    double qmax = 0, eps = 0;
    int64_t n_samples = 0;
    std::vector<double> Q;
    // runtime
    int status = 1;  // 1 pending / running, 0 done, < 0 error
    std::string why;  // the worker's message for a failed request
    std::vector<double> res;
    Clock::time_point t_submit, t_done;
    std::vector<GridEntry*> grids;  // per leaf
    size_t scratch_bytes = 0;
    void* scratch = nullptr;
    int stream = 0;
    cudaEvent_t done = nullptr;
    double* h_res = nullptr;
    void* h_stage = nullptr;  // pinned upload block of this request
    size_t h_stage_cap = 0;
};

// Pinned host blocks recycled once the device work that reads them is done.
// A block is taken (handed out, not yet returned), cooling (returned, its
// event not yet complete) or free.
struct PinnedPool {
    struct Block {
        void* p;
        size_t cap;
        bool taken;
        cudaEvent_t ev;  // cooling until it completes; null when free
    };
    std::vector<Block> blocks;
    ~PinnedPool() {
        for (Block& b : blocks) {
            if (b.ev) cudaEventDestroy(b.ev);
            cudaFreeHost(b.p);
        }
    }
    void* get(size_t n, size_t* cap) {
        for (Block& b : blocks) {
            if (b.taken || b.cap < n) continue;
            if (b.ev) {
                if (cudaEventQuery(b.ev) != cudaSuccess) continue;
                cudaEventDestroy(b.ev);
                b.ev = nullptr;
            }
            b.taken = true;
            *cap = b.cap;
            return b.p;
        }
        size_t c = 64 << 10;
        while (c < n) c <<= 1;
        void* p = nullptr;
        if (cudaMallocHost(&p, c) != cudaSuccess) return nullptr;
        blocks.push_back({p, c, true, nullptr});
        *cap = c;
        return p;
    }
    // The block is reusable after the work queued on s so far completes.
    void put(void* p, cudaStream_t s) {
        for (Block& b : blocks)
            if (b.p == p && b.taken) {
                b.taken = false;
                cudaEvent_t ev = nullptr;
                if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess &&
                    cudaEventRecord(ev, s) == cudaSuccess) {
                    b.ev = ev;
                } else {
                    if (ev) cudaEventDestroy(ev);
                    cudaStreamSynchronize(s);
                }
                return;
            }
    }
};

}  // namespace

struct dpx_server_s {
    dpx_ctx ctx = nullptr;
    int64_t budget = 0;
    int max_inflight = 1;
    std::vector<cudaStream_t> streams;
    cudaStream_t fill_stream = nullptr;
    double* d_dirs = nullptr;
    int64_t n_dirs = 0;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stopping = false;
    uint64_t next_ticket = 1;
    std::deque<Request*> pending;
    std::list<Request*> inflight;
    std::unordered_map<uint64_t, Request*> by_ticket;
    std::unordered_map<uint64_t, GridEntry*> cache;
    uint64_t use_clock = 0;
    int next_stream = 0;
    PinnedPool pinned;
    dpx_server_stats st{};
    std::vector<char> host;  // staging scratch (worker thread only)
};

namespace {

void entry_free(dpx_server_s* S, GridEntry* g) {
    if (g->cells) cudaFreeAsync(g->cells, S->fill_stream);
    if (g->ready) cudaEventDestroy(g->ready);
    S->st.bytes_in_use -= (int64_t)g->bytes;
    delete g;
}

// Frees unpinned cached grids, least recently used first, until `need` fits.
bool make_room(dpx_server_s* S, int64_t need) {
    while (S->st.bytes_in_use + need > S->budget) {
        GridEntry* victim = nullptr;
        uint64_t vkey = 0;
        for (auto& kv : S->cache)
            if (kv.second->pins == 0 && (!victim || kv.second->last_use < victim->last_use)) {
                victim = kv.second;
                vkey = kv.first;
            }
        if (!victim) return false;
        S->cache.erase(vkey);
        entry_free(S, victim);
        S->st.evictions++;
    }
    return true;
}

uint64_t grid_key(const LeafCopy& l, int grid_size, double qmax, int precision) {
    uint64_t h = l.key;
    h = fnv(h, &grid_size, sizeof grid_size);
    h = fnv(h, &qmax, sizeof qmax);
    h = fnv(h, &precision, sizeof precision);
    return h ? h : 1;
}

// Admission: pending requests in order; a request that does not fit lets later ones pass.
void admit_locked(dpx_server_s* S, std::vector<Request*>& admitted) {
    for (auto it = S->pending.begin(); it != S->pending.end();) {
        if ((int)S->inflight.size() + (int)admitted.size() >= S->max_inflight) break;
        Request* r = *it;
        const Geom G = dpx::make_geom(r->grid_size, r->qmax);
        const size_t gbytes = al16((size_t)G.P * cell_bytes(r->precision));
        int64_t need = (int64_t)r->scratch_bytes;
        std::vector<uint64_t> keys(r->leaves.size());
        for (size_t l = 0; l < r->leaves.size(); ++l) {
            keys[l] = grid_key(r->leaves[l], r->grid_size, r->qmax, r->precision);
            bool dup = false;
            for (size_t k = 0; k < l; ++k) dup |= keys[k] == keys[l];
            if (!dup && !S->cache.count(keys[l])) need += (int64_t)gbytes;
        }
        if (need > S->budget) {  // can never fit
            r->status = DPX_ERR_OOM;
            r->why = "the request needs more device memory than the server's budget";
            r->t_done = Clock::now();
            S->st.failed++;
            it = S->pending.erase(it);
            S->cv_done.notify_all();
            continue;
        }
        // pin what is already resident (one pin per leaf) before evicting for the rest
        std::vector<char> pre(r->leaves.size(), 0);
        for (size_t l = 0; l < r->leaves.size(); ++l) {
            auto f = S->cache.find(keys[l]);
            if (f != S->cache.end()) {
                f->second->pins++;
                pre[l] = 1;
            }
        }
        if (!make_room(S, need)) {
            for (size_t l = 0; l < r->leaves.size(); ++l)
                if (pre[l]) S->cache[keys[l]]->pins--;
            ++it;
            continue;
        }
        r->grids.assign(r->leaves.size(), nullptr);
        for (size_t l = 0; l < r->leaves.size(); ++l) {
            GridEntry* g;
            auto f = S->cache.find(keys[l]);
            if (pre[l]) {
                g = f->second;
                bool first = true;
                for (size_t k = 0; k < l; ++k) first &= keys[k] != keys[l];
                if (first && g->filled) S->st.grid_hits++;
            } else if (f != S->cache.end()) {  // a repeat of a leaf this request adds
                g = f->second;
                g->pins++;
            } else {
                g = new GridEntry;
                g->key = keys[l];
                g->grid_size = r->grid_size;
                g->qmax = r->qmax;
                g->precision = r->precision;
                g->G = G;
                g->bytes = gbytes;
                g->pins = 1;
                g->src = &r->leaves[l];
                S->cache[keys[l]] = g;
                S->st.bytes_in_use += (int64_t)gbytes;
            }
            g->last_use = ++S->use_clock;
            r->grids[l] = g;
        }
        S->st.bytes_in_use += (int64_t)r->scratch_bytes;
        S->st.bytes_peak = std::max(S->st.bytes_peak, S->st.bytes_in_use);
        admitted.push_back(r);
        it = S->pending.erase(it);
    }
}

void retire_locked(dpx_server_s* S) {
    for (auto it = S->inflight.begin(); it != S->inflight.end();) {
        Request* r = *it;
        const cudaError_t q = cudaEventQuery(r->done);
        if (q == cudaErrorNotReady) {
            ++it;
            continue;
        }
        if (q == cudaSuccess) {
            std::memcpy(r->res.data(), r->h_res, (size_t)r->nq * sizeof(double));
            r->status = DPX_OK;
            S->st.completed++;
        } else {
            r->status = cuda_fail(q, "request");
            r->why = dpx_last_error();
            S->st.failed++;
        }
        r->t_done = Clock::now();
        cudaEventDestroy(r->done);
        r->done = nullptr;
        S->pinned.put(r->h_stage, S->streams[r->stream]);
        r->h_stage = nullptr;
        for (GridEntry* g : r->grids) g->pins--;
        S->st.bytes_in_use -= (int64_t)r->scratch_bytes;
        it = S->inflight.erase(it);
        S->cv_done.notify_all();
    }
}

struct Upload {
    std::vector<char>& h;
    size_t put(const void* src, size_t n) {
        const size_t at = al16(h.size());
        h.resize(at + n);
        if (n) std::memcpy(h.data() + at, src, n);
        return at;
    }
};

// Counters updated outside the lock, merged into the stats under it.
struct Delta {
    int64_t fill_launches = 0, grid_fills = 0;
};

// Fill every new grid of this turn: one FP32 launch over all of them, FP64 one each.
int launch_fills(dpx_server_s* S, const std::vector<GridEntry*>& fresh, Delta& dl) {
    if (fresh.empty()) return DPX_OK;
    dpx_ctx ctx = S->ctx;
    cudaStream_t s = S->fill_stream;
    const int cpt32 = ctx->fill_cpt, threads = ctx->fill_threads;
    std::vector<char>& h = S->host;
    h.clear();
    std::vector<dpx_pdb_desc> descs(fresh.size());
    std::vector<LeafTables> lt(fresh.size());
    for (size_t j = 0; j < fresh.size(); ++j) {
        const GridEntry& g = *fresh[j];
        const LeafCopy& l = *g.src;
        dpx_pdb_desc& d = descs[j];
        d = dpx_pdb_desc{};
        d.n_atoms = (int64_t)l.atoms.size() / 4;
        d.atoms = l.atoms.data();
        d.n_ions = l.n_ions;
        d.atoms_per_ion = l.api.data();
        d.coeffs = l.coeffs.data();
        d.ion_rads = l.rads.data();
        d.flags = l.flags;
        d.solvent_ed = l.sol_ed;
        d.c1 = l.c1;
        d.scale = l.scale;
        d.center = l.has_center ? l.center : nullptr;
        d.n_boxes = (int64_t)l.boxes.size() / 8;
        d.boxes = l.boxes.empty() ? nullptr : l.boxes.data();
        d.voxel_step = l.voxel_step;
        const bool fp32 = g.precision == DPX_FP32;
        stage_leaf(h, d, g.G, fp32, fp32 ? cpt32 : dpx::kFill64Cells, lt[j]);
    }
    // the harmonic method plans the FP32 leaves it takes (on the fill stream;
    // this worker waits for the planning's device steps), the rest are staged
    // for one direct-sum launch
    std::vector<HarmPlan> plans(fresh.size());
    struct Release {
        std::vector<HarmPlan>& p;
        ~Release() {
            for (HarmPlan& x : p) harmonic_plan_release(x);
        }
    } release{plans};
    std::vector<char> harm(fresh.size(), 0);
    if (ctx->fill_method == DPX_FILL_HARMONIC)
        for (size_t j = 0; j < fresh.size(); ++j) {
            if (fresh[j]->precision != DPX_FP32) continue;
            const int rc = harmonic_plan(s, descs[j], fresh[j]->G, plans[j]);
            if (rc < 0) return rc;
            harm[j] = rc == DPX_OK;
        }
    const size_t jobs_at = al16(h.size());
    size_t n32 = 0;
    for (size_t j = 0; j < fresh.size(); ++j) n32 += fresh[j]->precision == DPX_FP32 && !harm[j];
    h.resize(jobs_at + n32 * sizeof(dpx::FillJob));
    const size_t counter_at = al16(h.size());
    h.resize(counter_at + 64, 0);
    // the harmonic fills' job table goes last; its room is counted before the
    // staging block is allocated
    size_t n_harm = 0;
    for (size_t j = 0; j < fresh.size(); ++j) n_harm += harm[j] != 0;
    const size_t hjobs_at = al16(h.size());
    h.resize(hjobs_at + n_harm * sizeof(dpx::HarmJob), 0);
    // device: grids, then one staging block (freed in stream order after the launches)
    for (GridEntry* g : fresh) DPX_CUDA(cudaMallocAsync(&g->cells, g->bytes, s));
    char* d = nullptr;
    DPX_CUDA(cudaMallocAsync((void**)&d, h.size(), s));
    std::vector<dpx::FillJob> jobs;
    int64_t tiles = 0;
    for (size_t j = 0; j < fresh.size(); ++j) {
        if (fresh[j]->precision != DPX_FP32 || harm[j]) continue;
        jobs.push_back(make_job(descs[j], lt[j], d, fresh[j]->G, fresh[j]->cells, tiles));
        tiles += (lt[j].items + threads - 1) / threads;
    }
    if (!jobs.empty()) std::memcpy(h.data() + jobs_at, jobs.data(), jobs.size() * sizeof(dpx::FillJob));
    // the harmonic fills' job table: one scratch block, each fill its own part
    std::vector<dpx::HarmJob> hj;
    size_t hscratch = 0;
    for (size_t j = 0; j < fresh.size(); ++j) {
        if (!harm[j]) continue;
        dpx::HarmJob J = harmonic_job(plans[j], hscratch, 0);
        J.grid_ptr = reinterpret_cast<float4*>(fresh[j]->cells);
        hj.push_back(J);
        hscratch += (plans[j].scratch_bytes + 255) & ~size_t(255);
    }
    const dpx::HarmShape hshape = dpx::plan_harmonic_jobs(hj.data(), (int)hj.size());
    if (hj.size() != n_harm) return fail(DPX_ERR_ARG, "harmonic job count changed while staging");
    if (!hj.empty()) std::memcpy(h.data() + hjobs_at, hj.data(), hj.size() * sizeof(dpx::HarmJob));
    size_t cap = 0;
    void* hp = S->pinned.get(h.size(), &cap);
    if (!hp) return fail(DPX_ERR_OOM, "pinned staging");
    std::memcpy(hp, h.data(), h.size());
    DPX_CUDA(cudaMemcpyAsync(d, hp, h.size(), cudaMemcpyHostToDevice, s));
    S->pinned.put(hp, s);
    bool boxes = false;
    for (const dpx::FillJob& J : jobs) boxes |= J.n_boxes > 0;
    cudaError_t e = dpx::launch_fill_f32_batch(s, reinterpret_cast<const dpx::FillJob*>(d + jobs_at), (int)jobs.size(),
                                               tiles, reinterpret_cast<unsigned long long*>(d + counter_at), cpt32,
                                               threads, ctx->fill_poly, ctx->fill_persistent, boxes);
    if (e != cudaSuccess) return cuda_fail(e, "fill launch");
    if (!jobs.empty()) dl.fill_launches++;
    for (size_t j = 0; j < fresh.size(); ++j) {
        if (fresh[j]->precision != DPX_FP64) continue;
        e = launch_leaf_f64(s, descs[j], lt[j], d, fresh[j]->G, fresh[j]->cells);
        if (e != cudaSuccess) return cuda_fail(e, "fill launch");
        dl.fill_launches++;
    }
    if (!hj.empty()) {  // the harmonic fills: four launches over their job table
        char* scratch = nullptr;
        DPX_CUDA(cudaMallocAsync((void**)&scratch, hscratch, s));
        e = dpx::launch_harmonic_jobs(s, reinterpret_cast<const dpx::HarmJob*>(d + hjobs_at), (int)hj.size(), hshape,
                                      scratch, nullptr, nullptr);
        cudaFreeAsync(scratch, s);
        if (e != cudaSuccess) return cuda_fail(e, "harmonic fill launch");
        dl.fill_launches += (hshape.moments > 0) + (hshape.groups > 0) +
                            (hshape.contract > 0) + (hshape.synth > 0);
    }
    DPX_CUDA(cudaFreeAsync(d, s));
    for (size_t j = 0; j < fresh.size(); ++j) {
        GridEntry* g = fresh[j];
        e = harm[j] ? cudaSuccess  // the harmonic synthesis writes the phi-spline derivatives
            : g->precision == DPX_FP32 ? dpx::launch_splines_f32(s, g->G, reinterpret_cast<float4*>(g->cells))
                                       : dpx::launch_splines_f64(s, g->G, reinterpret_cast<double4_32a*>(g->cells));
        if (e != cudaSuccess) return cuda_fail(e, "splines launch");
        DPX_CUDA(cudaEventCreateWithFlags(&g->ready, cudaEventDisableTiming));
        DPX_CUDA(cudaEventRecord(g->ready, s));
        g->filled = true;
        g->src = nullptr;  // the leaf copy belongs to a request and may go
        dl.grid_fills++;
    }
    return DPX_OK;
}

// One request's orientation average on its stream.
int launch_request(dpx_server_s* S, Request* r) {
    cudaStream_t s = S->streams[r->stream];
    const Geom G = dpx::make_geom(r->grid_size, r->qmax);
    const int nm = (int)r->model_leaf.size();
    std::vector<const void*> cells(nm);
    for (int m = 0; m < nm; ++m) cells[m] = r->grids[r->model_leaf[m]]->cells;
    for (GridEntry* g : r->grids) DPX_CUDA(cudaStreamWaitEvent(s, g->ready, 0));
    ModelTables T;
    if (int rc = build_models(nm, cells.data(), r->rot.data(), r->tr.data(), r->n_copies.data(),
                              r->copy_rot.empty() ? nullptr : r->copy_rot.data(),
                              r->copy_tr.empty() ? nullptr : r->copy_tr.data(), r->sym_scale.data(), T))
        return rc;
    Brackets B;
    make_brackets(G, r->grid_size, r->qmax, r->nq, r->Q.data(), B);
    dpx::AvgPlan P{};
    P.n_brackets = (int)B.layer.size();
    P.max_q = B.max_q;
    P.n_samples = r->n_samples;
    P.chunk = r->eps > 0.0 ? 100 : 128;
    P.chunk_off = r->eps > 0.0 ? 99 : 0;
    P.n_chunks = (r->n_samples + P.chunk_off + P.chunk - 1) / P.chunk;
    P.dir_stride = 0;
    P.dirs = S->d_dirs;
    P.need_dir = 0;
    for (const dpx::ModelDev& M : T.md)
        if (!M.plain || M.n_groups > 0) P.need_dir = 1;
    P.one_leaf = (nm == 1 && T.md[0].n_groups == 0) ? 1 : 0;
    std::vector<char> h;
    Upload U{h};
    const size_t oG = U.put(T.gstage.data(), T.gstage.size());
    const size_t oQ = U.put(B.q.data(), B.q.size() * sizeof(double));
    const size_t oL = U.put(B.layer.data(), B.layer.size() * sizeof(int));
    const size_t oO = U.put(B.off.data(), B.off.size() * sizeof(int));
    const size_t oI = U.put(B.qidx.data(), B.qidx.size() * sizeof(int));
    const size_t oM = al16(h.size());
    h.resize(oM + T.md.size() * sizeof(dpx::ModelDev));
    const size_t oR = al16(h.size());
    h.resize(oR + (size_t)r->nq * sizeof(double));
    const size_t oP = al16(h.size());
    const size_t part = ((size_t)P.n_brackets * P.n_chunks + (size_t)P.n_brackets * 5) * P.max_q * sizeof(double);
    // with eps = 0 the shared directions are taken in angular order
    const size_t oS = al16(oP + part);
    const size_t sort_bytes = r->eps == 0.0 ? dpx::dir_sort_bytes(r->n_samples) : 0;
    const size_t total = oS + sort_bytes + 64;
    char* d = nullptr;
    DPX_CUDA(cudaMallocAsync((void**)&d, total, s));
    place_models(T, d + oG);
    std::memcpy(h.data() + oM, T.md.data(), T.md.size() * sizeof(dpx::ModelDev));
    P.br_q = reinterpret_cast<const double*>(d + oQ);
    P.br_layer = reinterpret_cast<const int*>(d + oL);
    P.br_q_off = reinterpret_cast<const int*>(d + oO);
    P.br_qidx = reinterpret_cast<const int*>(d + oI);
    P.partial = reinterpret_cast<double*>(d + oP);
    P.sort_scratch = sort_bytes ? reinterpret_cast<int*>(d + oS) : nullptr;
    size_t cap = 0;
    const size_t stage = oR + (size_t)r->nq * sizeof(double);
    char* hp = static_cast<char*>(S->pinned.get(stage, &cap));
    if (!hp) return fail(DPX_ERR_OOM, "pinned staging");
    r->h_stage = hp;
    r->h_stage_cap = cap;
    std::memcpy(hp, h.data(), oR);
    r->h_res = reinterpret_cast<double*>(hp + oR);
    double* d_res = reinterpret_cast<double*>(d + oR);
    DPX_CUDA(cudaMemcpyAsync(d, hp, oR, cudaMemcpyHostToDevice, s));
    DPX_CUDA(cudaMemsetAsync(d_res, 0, (size_t)r->nq * sizeof(double), s));
    const bool fp64 = r->precision == DPX_FP64;
    const dpx::ModelDev* d_models = reinterpret_cast<const dpx::ModelDev*>(d + oM);
    cudaError_t e = dpx::launch_average(s, fp64, G, nm, d_models, P);
    if (e == cudaSuccess) e = dpx::launch_finalize(s, P, r->eps, d_res);
    if (e == cudaSuccess && r->Q[0] == 0.0) e = dpx::launch_origin_models(s, fp64, d_models, nm, d_res);
    if (e != cudaSuccess) return cuda_fail(e, "average launch");
    DPX_CUDA(cudaMemcpyAsync(r->h_res, d_res, (size_t)r->nq * sizeof(double), cudaMemcpyDeviceToHost, s));
    DPX_CUDA(cudaFreeAsync(d, s));
    DPX_CUDA(cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming));
    DPX_CUDA(cudaEventRecord(r->done, s));
    return DPX_OK;
}

void worker_main(dpx_server_s* S) {
    cudaSetDevice(S->ctx->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        retire_locked(S);
        if (S->stopping && S->pending.empty() && S->inflight.empty()) break;
        std::vector<Request*> admitted;
        admit_locked(S, admitted);
        if (admitted.empty()) {
            S->cv_work.wait_for(lk, std::chrono::microseconds(S->inflight.empty() ? 5000 : 50));
            continue;
        }
        S->st.steps++;
        std::vector<GridEntry*> fresh;
        for (Request* r : admitted)
            for (GridEntry* g : r->grids)
                if (!g->filled && std::find(fresh.begin(), fresh.end(), g) == fresh.end()) fresh.push_back(g);
        for (Request* r : admitted) {
            r->stream = S->next_stream;
            S->next_stream = (S->next_stream + 1) % (int)S->streams.size();
            S->inflight.push_back(r);
        }
        lk.unlock();  // device work outside the lock: submitters keep queueing
        Delta dl;
        int rc = launch_fills(S, fresh, dl);
        std::vector<int> rcs(admitted.size(), rc);
        std::vector<std::string> why(admitted.size(), rc ? std::string(dpx_last_error()) : std::string());
        for (size_t k = 0; k < admitted.size(); ++k)
            if (!rc) {
                rcs[k] = launch_request(S, admitted[k]);
                if (rcs[k]) why[k] = dpx_last_error();
            }
        lk.lock();
        S->st.fill_launches += dl.fill_launches;
        S->st.grid_fills += dl.grid_fills;
        bool any_failed = false;
        for (size_t k = 0; k < admitted.size(); ++k) {
            Request* r = admitted[k];
            if (rcs[k] == DPX_OK) continue;
            // could not be queued: drain its stream, release it now
            any_failed = true;
            cudaStreamSynchronize(S->streams[r->stream]);
            if (r->done) cudaEventDestroy(r->done);
            r->done = nullptr;
            if (r->h_stage) S->pinned.put(r->h_stage, S->streams[r->stream]);
            r->h_stage = nullptr;
            for (GridEntry* g : r->grids) g->pins--;
            S->st.bytes_in_use -= (int64_t)r->scratch_bytes;
            S->inflight.remove(r);
            r->status = rcs[k];
            r->why = why[k];
            r->t_done = Clock::now();
            S->st.failed++;
        }
        if (any_failed) {  // grids whose fill never got queued leave the cache
            cudaStreamSynchronize(S->fill_stream);
            for (GridEntry* g : fresh)
                if (!g->filled && g->pins == 0) {
                    S->cache.erase(g->key);
                    entry_free(S, g);
                }
            S->cv_done.notify_all();
        }
    }
}

}  // namespace

extern "C" {

int dpx_server_create(dpx_ctx ctx, int64_t hbm_budget_bytes, int max_inflight, int n_streams, const double* dirs,
                      int64_t n_dirs, dpx_server* out) {
    if (!ctx || !dirs || n_dirs <= 0 || !out) return fail(DPX_ERR_ARG, "NULL or empty argument");
    if (max_inflight <= 0 || n_streams <= 0 || n_streams > 64) return fail(DPX_ERR_ARG, "bad slot counts");
    if (int rc = set_device(ctx)) return rc;
    if (hbm_budget_bytes <= 0) {
        size_t fr = 0, tot = 0;
        DPX_CUDA(cudaMemGetInfo(&fr, &tot));
        hbm_budget_bytes = (int64_t)(fr * 0.8);
    }
    auto* S = new dpx_server_s;
    S->ctx = ctx;
    ctx_retain(ctx);
    S->budget = hbm_budget_bytes;
    S->st.budget = hbm_budget_bytes;
    S->max_inflight = max_inflight;
    S->n_dirs = n_dirs;
    cudaError_t e = cudaStreamCreateWithFlags(&S->fill_stream, cudaStreamNonBlocking);
    for (int k = 0; k < n_streams && e == cudaSuccess; ++k) {
        cudaStream_t st = nullptr;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) S->streams.push_back(st);
    }
    if (e == cudaSuccess) e = cudaMalloc((void**)&S->d_dirs, (size_t)n_dirs * 2 * sizeof(double));
    if (e == cudaSuccess)
        e = cudaMemcpy(S->d_dirs, dirs, (size_t)n_dirs * 2 * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        const int rc = cuda_fail(e, "server setup");
        for (cudaStream_t st : S->streams) cudaStreamDestroy(st);
        if (S->fill_stream) cudaStreamDestroy(S->fill_stream);
        if (S->d_dirs) cudaFree(S->d_dirs);
        ctx_release(ctx);
        delete S;
        return rc;
    }
    S->worker = std::thread(worker_main, S);
    *out = S;
    return DPX_OK;
}

int dpx_server_submit(dpx_server S, const dpx_request* q, uint64_t* ticket) {
    if (!S || !q || !ticket) return fail(DPX_ERR_ARG, "NULL argument");
    if (q->n_leaves <= 0 || !q->leaves || q->n_models <= 0 || !q->model_leaf)
        return fail(DPX_ERR_ARG, "a request needs leaves and models");
    if (q->precision != DPX_FP32 && q->precision != DPX_FP64) return fail(DPX_ERR_ARG, "bad precision");
    if (q->grid_size < 2 || (q->grid_size & 1) || !(q->qmax > 0)) return fail(DPX_ERR_ARG, "bad grid");
    if (q->nq <= 0 || !q->Q) return fail(DPX_ERR_ARG, "no q values");
    for (int k = 1; k < q->nq; ++k)
        if (!(q->Q[k] >= q->Q[k - 1])) return fail(DPX_ERR_ARG, "Q must be ascending");
    if (q->Q[0] < 0 || q->Q[q->nq - 1] > q->qmax * (1.0 + 1e-12)) return fail(DPX_ERR_ARG, "q outside [0, qmax]");
    if (q->n_samples <= 0 || q->n_samples > S->n_dirs)
        return fail(DPX_ERR_ARG, "n_samples must be in [1, %lld]", (long long)S->n_dirs);
    auto* r = new Request;
    r->leaves.resize(q->n_leaves);
    for (int l = 0; l < q->n_leaves; ++l) {
        const dpx_pdb_desc& d = q->leaves[l];
        if (int rc = check_pdb(d)) {
            delete r;
            return rc;
        }
        if (d.atoms_on_device) {
            delete r;
            return fail(DPX_ERR_ARG, "server requests take host atoms");
        }
        if (d.aff) {
            delete r;
            return fail(DPX_ERR_ARG, "server requests take leaves with form-factor coefficients");
        }
        LeafCopy& c = r->leaves[l];
        c.atoms.assign(d.atoms, d.atoms + 4 * d.n_atoms);
        c.api.assign(d.atoms_per_ion, d.atoms_per_ion + d.n_ions);
        c.coeffs.assign(d.coeffs, d.coeffs + 9 * d.n_ions);
        c.rads.assign(d.ion_rads, d.ion_rads + d.n_ions);
        c.n_ions = d.n_ions;
        c.flags = d.flags;
        c.sol_ed = d.solvent_ed;
        c.c1 = d.c1;
        c.scale = d.scale;
        c.has_center = d.center != nullptr;
        if (d.center)
            for (int k = 0; k < 3; ++k) c.center[k] = d.center[k];
        if (d.n_boxes > 0 && d.boxes) c.boxes.assign(d.boxes, d.boxes + 8 * d.n_boxes);
        c.voxel_step = d.voxel_step;
        uint64_t h = q->leaf_keys && q->leaf_keys[l] ? q->leaf_keys[l] : 0;
        if (!h) {  // content key
            h = 1469598103934665603ull;
            h = fnv(h, c.atoms.data(), c.atoms.size() * sizeof(float));
            h = fnv(h, c.api.data(), c.api.size() * sizeof(int));
            h = fnv(h, c.coeffs.data(), c.coeffs.size() * sizeof(double));
            h = fnv(h, c.rads.data(), c.rads.size() * sizeof(double));
            const double p[4] = {c.sol_ed, c.c1, c.scale, (double)c.flags};
            h = fnv(h, p, sizeof p);
            if (c.has_center) h = fnv(h, c.center, sizeof c.center);
            h = fnv(h, c.boxes.data(), c.boxes.size() * sizeof(float));
            h = fnv(h, &c.voxel_step, sizeof c.voxel_step);
        }
        c.key = h;
    }
    const int nm = q->n_models;
    r->model_leaf.assign(q->model_leaf, q->model_leaf + nm);
    for (int m = 0; m < nm; ++m)
        if (r->model_leaf[m] < 0 || r->model_leaf[m] >= q->n_leaves) {
            delete r;
            return fail(DPX_ERR_ARG, "model %d names leaf %d", m, r->model_leaf[m]);
        }
    r->rot.assign(3 * nm, 0.0);
    r->tr.assign(3 * nm, 0.0);
    r->n_copies.assign(nm, 0);
    r->sym_scale.assign(nm, 1.0);
    if (q->rot) r->rot.assign(q->rot, q->rot + 3 * nm);
    if (q->tr) r->tr.assign(q->tr, q->tr + 3 * nm);
    if (q->sym_scale) r->sym_scale.assign(q->sym_scale, q->sym_scale + nm);
    int64_t copies = 0;
    if (q->n_copies) {
        r->n_copies.assign(q->n_copies, q->n_copies + nm);
        for (int m = 0; m < nm; ++m) {
            if (r->n_copies[m] < 0) {
                delete r;
                return fail(DPX_ERR_ARG, "negative copy count");
            }
            copies += r->n_copies[m];
        }
        if (copies > 0 && (!q->copy_rot || !q->copy_tr)) {
            delete r;
            return fail(DPX_ERR_ARG, "copies need copy_rot and copy_tr");
        }
        if (copies > 0) {
            r->copy_rot.assign(q->copy_rot, q->copy_rot + 3 * copies);
            r->copy_tr.assign(q->copy_tr, q->copy_tr + 3 * copies);
        }
    }
    r->grid_size = q->grid_size;
    r->qmax = q->qmax;
    r->precision = q->precision;
    r->nq = q->nq;
    r->Q.assign(q->Q, q->Q + q->nq);
    r->n_samples = q->n_samples;
    r->eps = q->eps;
    r->res.assign(q->nq, 0.0);
    // device scratch of the average: tables + partial sums + result
    {
        const Geom G = dpx::make_geom(r->grid_size, r->qmax);
        Brackets B;
        make_brackets(G, r->grid_size, r->qmax, r->nq, r->Q.data(), B);
        const int chunk = r->eps > 0.0 ? 100 : 128, off = r->eps > 0.0 ? 99 : 0;
        const int64_t n_chunks = (r->n_samples + off + chunk - 1) / chunk;
        const size_t tables = 9 * sizeof(double) * (size_t)copies + 3 * sizeof(double) * (size_t)copies +
                              sizeof(int) * ((size_t)copies + (size_t)nm) + nm * sizeof(dpx::ModelDev) +
                              B.q.size() * (sizeof(double) + sizeof(int)) + 2 * B.layer.size() * sizeof(int) + 1024;
        r->scratch_bytes = al16(tables) + al16((size_t)r->nq * sizeof(double)) +
                           ((size_t)B.layer.size() * n_chunks + B.layer.size() * 5) * B.max_q * sizeof(double) + 256 +
                           (r->eps == 0.0 ? dpx::dir_sort_bytes(r->n_samples) : 0);
    }
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> g(S->mu);
        if (S->stopping) {
            delete r;
            return fail(DPX_ERR_ARG, "server is stopping");
        }
        r->ticket = S->next_ticket++;
        S->by_ticket[r->ticket] = r;
        S->pending.push_back(r);
        S->st.submitted++;
        *ticket = r->ticket;
    }
    S->cv_work.notify_one();
    return DPX_OK;
}

int dpx_server_poll(dpx_server S, uint64_t ticket) {
    if (!S) return fail(DPX_ERR_ARG, "server is NULL");
    std::lock_guard<std::mutex> g(S->mu);
    auto f = S->by_ticket.find(ticket);
    if (f == S->by_ticket.end()) return fail(DPX_ERR_ARG, "unknown ticket");
    return f->second->status == 1 ? 0 : 1;
}

int dpx_server_wait(dpx_server S, uint64_t ticket, double* res, double* latency_ms) {
    if (!S) return fail(DPX_ERR_ARG, "server is NULL");
    Request* r = nullptr;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        auto f = S->by_ticket.find(ticket);
        if (f == S->by_ticket.end()) return fail(DPX_ERR_ARG, "unknown ticket");
        r = f->second;
        S->cv_done.wait(lk, [&] { return r->status != 1; });
        S->by_ticket.erase(f);
    }
    const int status = r->status;
    if (status == DPX_OK && res) std::memcpy(res, r->res.data(), r->res.size() * sizeof(double));
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    const std::string why = r->why;
    delete r;
    if (status != DPX_OK) return fail(status, "request failed (status %d): %s", status, why.c_str());
    return DPX_OK;
}

int dpx_server_stats_get(dpx_server S, dpx_server_stats* st) {
    if (!S || !st) return fail(DPX_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(S->mu);
    *st = S->st;
    st->cached_grids = (int64_t)S->cache.size();
    return DPX_OK;
}

int dpx_server_destroy(dpx_server S) {
    if (!S) return fail(DPX_ERR_ARG, "server is NULL");
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->stopping = true;
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    set_device(S->ctx);
    cudaStreamSynchronize(S->fill_stream);
    for (cudaStream_t st : S->streams) cudaStreamSynchronize(st);
    for (auto& kv : S->cache) {
        if (kv.second->cells) cudaFreeAsync(kv.second->cells, S->fill_stream);
        if (kv.second->ready) cudaEventDestroy(kv.second->ready);
        delete kv.second;
    }
    cudaStreamSynchronize(S->fill_stream);
    for (auto& kv : S->by_ticket) delete kv.second;  // finished but never collected
    for (cudaStream_t st : S->streams) cudaStreamDestroy(st);
    cudaStreamDestroy(S->fill_stream);
    cudaFree(S->d_dirs);
    dpx_ctx ctx = S->ctx;
    delete S;
    ctx_release(ctx);
    return DPX_OK;
}

}  // extern "C"
