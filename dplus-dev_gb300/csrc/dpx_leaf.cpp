// dpx_leaf.cpp — prepared leaves: the reference's PDBAmplitude after
// PreCalculate (Backend/Backend/PDBAmplitude.cpp:1199-1336), i.e. everything
// about a leaf that does not change from one grid fill to the next, done once.
//
// dpx_leaf_create plans the fill of one grid: the harmonic fill's plan (FP32
// with the harmonic method: point sets grouped, voxels binned, tables, in
// device memory the leaf owns, plus its launch scratch) or the direct sum's
// staged tables (FP32 direct, FP64).  dpx_leaf_fill then only queues kernels on
// the context's stream: no host work, no copies from the host, no
// synchronization (its side stream forks from and joins back into the
// context's stream by events), so a stream capture can record it.
#include "dpx_host.h"

#include <cstring>
#include <vector>

using namespace dpxh;

struct dpx_leaf_s {
    dpx_ctx ctx = nullptr;
    dpx_grid grid = nullptr;
    bool harmonic = false;
    HarmPlan plan;
    void* scratch = nullptr;   // the harmonic fill's launch scratch
    void* tables = nullptr;    // the direct sum's staged tables (+ job table and tile counter)
    LeafTables lt;
    dpx_pdb_desc d{};          // scalars of the leaf; device atoms pointer when they are the caller's
    size_t o_jobs = 0, o_counter = 0, table_bytes = 0;
    int64_t tiles = 0;
    int cpt = 8, threads = 128, poly = 0;
    bool persistent = false;
};

namespace {

void leaf_free(dpx_leaf L) {
    if (!L) return;
    set_device(L->ctx);
    harmonic_plan_release(L->plan);
    cudaStreamSynchronize(L->ctx->stream);
    if (L->scratch) cudaFree(L->scratch);
    if (L->tables) cudaFree(L->tables);
    ctx_release(L->ctx);
    delete L;
}

}  // namespace

extern "C" {

int dpx_leaf_create(dpx_grid g, const dpx_pdb_desc* d, dpx_leaf* out) {
    if (!g || !d || !out) return fail(DPX_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (int rc = check_pdb(*d)) return rc;
    if (int rc = check_leaf_grid(*d, g->g)) return rc;
    dpx_ctx ctx = g->ctx;
    if (int rc = set_device(ctx)) return rc;
    auto* L = new dpx_leaf_s;
    L->ctx = ctx;
    ctx_retain(ctx);
    L->grid = g;
    L->d = *d;
    cudaStream_t s = ctx->stream;
    const bool fp32 = g->precision == DPX_FP32;
    if (fp32 && ctx->fill_method == DPX_FILL_HARMONIC) {
        const int rc = harmonic_plan(s, *d, g->g, L->plan);
        if (rc < 0) {
            leaf_free(L);
            return rc;
        }
        L->harmonic = rc == DPX_OK;
    }
    int rc = DPX_OK;
    if (L->harmonic) {
        HarmStreams hs;  // creates the timing events now, outside any capture
        rc = ctx_harmonic_streams(ctx, hs);
        cudaError_t e = rc ? cudaSuccess : cudaMalloc(&L->scratch, L->plan.scratch_bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            rc = fail(DPX_ERR_OOM, "harmonic fill needs %zu bytes of scratch (%s)", L->plan.scratch_bytes,
                      cudaGetErrorString(e));
        }
    } else {
        // the direct sum's tables, staged once; the job table points at the grid
        L->cpt = fp32 ? ctx->fill_cpt : dpx::kFill64Cells;
        L->threads = ctx->fill_threads;
        L->poly = ctx->fill_poly;
        L->persistent = ctx->fill_persistent;
        std::vector<char> h;
        stage_leaf(h, *d, g->g, fp32, L->cpt, L->lt);
        L->o_jobs = al16(h.size());
        L->o_counter = al16(L->o_jobs + sizeof(dpx::FillJob));
        h.resize(L->o_counter + 64, 0);
        L->table_bytes = h.size();
        cudaError_t e = cudaMalloc(&L->tables, h.size());
        if (e == cudaSuccess && fp32) {
            const dpx::FillJob J = make_job(*d, L->lt, static_cast<const char*>(L->tables), g->g, g->cells, 0);
            std::memcpy(h.data() + L->o_jobs, &J, sizeof J);
            L->tiles = (L->lt.items + L->threads - 1) / L->threads;
        }
        if (e == cudaSuccess) e = cudaMemcpy(L->tables, h.data(), h.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_fail(e, "leaf tables");
        // host atoms are read only here: the staged copy serves every fill
        if (!d->atoms_on_device) L->d.atoms = nullptr;
        L->d.boxes = nullptr;
    }
    if (!rc) {
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_fail(e, "leaf preparation");
    }
    if (rc) {
        leaf_free(L);
        return rc;
    }
    *out = L;
    return DPX_OK;
}

int dpx_leaf_fill(dpx_leaf L) {
    if (!L) return fail(DPX_ERR_ARG, "leaf is NULL");
    dpx_ctx ctx = L->ctx;
    if (int rc = set_device(ctx)) return rc;
    cudaStream_t s = ctx->stream;
    dpx_grid g = L->grid;
    g->splines_current = false;
    if (L->harmonic) {
        HarmStreams hs;
        if (int rc = ctx_harmonic_streams(ctx, hs)) return rc;
        if (int rc = harmonic_launch(hs, L->plan, L->scratch, reinterpret_cast<float4*>(g->cells))) return rc;
        ctx_stage_record(ctx, L->plan);
        g->splines_current = true;  // the synthesis wrote the phi-spline derivatives
        return DPX_OK;
    }
    const char* A = static_cast<const char*>(L->tables);
    cudaError_t e;
    if (g->precision == DPX_FP32) {
        e = dpx::launch_fill_f32_batch(s, reinterpret_cast<const dpx::FillJob*>(A + L->o_jobs), 1, L->tiles,
                                       reinterpret_cast<unsigned long long*>(const_cast<char*>(A) + L->o_counter),
                                       L->cpt, L->threads, L->poly, L->persistent, L->lt.n_boxes > 0);
        if (e == cudaSuccess) e = dpx::launch_splines_f32(s, g->g, reinterpret_cast<float4*>(g->cells));
    } else {
        e = launch_leaf_f64(s, L->d, L->lt, A, g->g, g->cells);
        if (e == cudaSuccess) e = dpx::launch_splines_f64(s, g->g, reinterpret_cast<double4_32a*>(g->cells));
    }
    if (e != cudaSuccess) return cuda_fail(e, "leaf fill");
    g->splines_current = true;
    return DPX_OK;
}

int dpx_leaf_info(dpx_leaf L, int* harmonic, int64_t* launches, int64_t* device_bytes) {
    if (!L) return fail(DPX_ERR_ARG, "leaf is NULL");
    if (harmonic) *harmonic = L->harmonic ? 1 : 0;
    if (launches) *launches = L->harmonic ? harmonic_launches(L->plan) : 2;
    if (device_bytes)
        *device_bytes = (int64_t)(L->harmonic ? L->plan.arena_bytes + L->plan.scratch_bytes : L->table_bytes);
    return DPX_OK;
}

int dpx_leaf_destroy(dpx_leaf L) {
    if (!L) return fail(DPX_ERR_ARG, "leaf is NULL");
    leaf_free(L);
    return DPX_OK;
}

}  // extern "C"
