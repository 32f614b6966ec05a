// dpx_api.cpp — host side of libdpx: the C-ABI (include/dpx.h), device-resident
// grids, form-factor tables, bracket plans and the drop-in wrappers with the
// reference's argument meaning.  No entry point throws or traps; failures are
// status codes with a per-thread message.
#include "dpx_host.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include <unordered_map>

using dpx::Geom;
using namespace dpxh;

namespace dpxh {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(DPX_ERR_OOM, "%s: %s", where, cudaGetErrorString(e));
    }
    return fail(DPX_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

}  // namespace dpxh

namespace dpxh {

int set_device(dpx_ctx ctx) {
    int cur = -1;
    DPX_CUDA(cudaGetDevice(&cur));
    if (cur != ctx->device) DPX_CUDA(cudaSetDevice(ctx->device));
    return DPX_OK;
}

size_t cell_bytes(int precision) { return precision == DPX_FP64 ? sizeof(double4_32a) : sizeof(float4); }

// FP32 fill launch shapes the autotuner sweeps: {cells per work item, threads
// per block (= atoms per shared-memory tile), persistent schedule, columns
// whose sincos run on the FMA pipe}; flat and persistent forms pairwise; the
// row {0, 0, 0, 0} stands for the harmonic method.
extern const int kFillShape[][4] = {{2, 256, 0, 0}, {2, 256, 1, 0}, {4, 128, 0, 0}, {4, 128, 1, 0}, {4, 256, 0, 0},
                                    {4, 256, 1, 0}, {6, 128, 0, 0}, {6, 128, 1, 0}, {6, 256, 0, 0}, {6, 256, 1, 0},
                                    {8, 128, 0, 0}, {8, 128, 1, 0}, {8, 256, 0, 0}, {8, 256, 1, 0}, {8, 128, 0, 1},
                                    {8, 128, 1, 1}, {8, 128, 0, 2}, {8, 128, 1, 2}, {8, 128, 0, 3}, {8, 128, 1, 3},
                                    {0, 0, 0, 0}};  // the last row: the harmonic method
extern const int kFillShapes = 21;

// Unique-ion form factors minus the Gaussian dummy-atom solvent
// (Atomic Form Factor.cpp:91-115, 121-176; r_m :11-27) for shells 0..Lp,
// layout [U][Lp+1].
void aff_at(int U, const int* api, const double* coeffs, const double* rads, int flags, double sol_ed, double c1,
            int nq, const double* qs, std::vector<double>& out) {
    double s3 = 0, n = 0;
    for (int u = 0; u < U; ++u) {
        s3 += rads[u] * rads[u] * rads[u] * api[u];
        n += api[u];
    }
    const double rm = std::cbrt(s3 / n);
    out.assign((size_t)U * nq, 0.0);
    for (int l = 0; l < nq; ++l) {
        const double q = qs[l];
        const double s2 = q * q / (100.0 * 157.913670417429737901351855998);
        for (int u = 0; u < U; ++u) {
            double f = 0;
            if (flags & DPX_CALC_ATOMIC_FORMFACTORS) {
                for (int k = 0; k < 4; ++k) f += coeffs[u + 2 * k * U] * std::exp(-s2 * coeffs[u + (2 * k + 1) * U]);
                f += coeffs[u + 8 * U];
            }
            double solvent = 0;
            if (flags & DPX_CALC_DUMMY_SOLVENT) {
                const double r = rads[u];
                solvent = 4.1887902047863909846 * r * r * r * std::exp(-(rm * rm) * (q * q) * 0.2067834969664667) *
                          sol_ed * c1 * c1 * c1 *
                          std::exp(-0.6822178052976590 * q * q * rm * rm * (c1 * c1 - 1.0));
            }
            out[(size_t)u * nq + l] = f - solvent;
        }
    }
}

void aff_table(int U, const int* api, const double* coeffs, const double* rads, int flags, double sol_ed,
               double c1, int Lp, double step, std::vector<double>& out) {
    std::vector<double> q(Lp + 1);
    for (int l = 0; l <= Lp; ++l) q[l] = l * step;
    aff_at(U, api, coeffs, rads, flags, sol_ed, c1, Lp + 1, q.data(), out);
}

void leaf_aff_table(const dpx_pdb_desc& d, int Lp, double step, std::vector<double>& out) {
    if (!d.aff) {
        aff_table(d.n_ions, d.atoms_per_ion, d.coeffs, d.ion_rads, d.flags, d.solvent_ed, d.c1, Lp, step, out);
        return;
    }
    out.assign((size_t)d.n_ions * (Lp + 1), 0.0);
    for (int u = 0; u < d.n_ions; ++u)
        for (int k = 0; k <= Lp && k < d.aff_n; ++k) out[(size_t)u * (Lp + 1) + k] = d.aff[(size_t)u * d.aff_n + k];
}

int check_leaf_grid(const dpx_pdb_desc& d, const dpx::Geom& G) {
    if (d.aff && d.aff_n < G.Lp + 1)
        return fail(DPX_ERR_ARG, "the tabulated form factors cover %d shells; the grid has %d", d.aff_n, G.Lp + 1);
    return DPX_OK;
}

// Tait-Bryan X1Y2Z3 rotation (the reference's EulerD, Amplitude.h:557-573).
void euler(double a, double b, double c, double R[9]) {
    const double c1 = std::cos(a), s1 = std::sin(a), c2 = std::cos(b), s2 = std::sin(b), c3 = std::cos(c),
                 s3 = std::sin(c);
    R[0] = c2 * c3; R[1] = -c2 * s3; R[2] = s2;
    R[3] = c1 * s3 + c3 * s1 * s2; R[4] = c1 * c3 - s1 * s2 * s3; R[5] = -c2 * s1;
    R[6] = s1 * s3 - c1 * c3 * s2; R[7] = c3 * s1 + c1 * s2 * s3; R[8] = c1 * c2;
}

}  // namespace dpxh

int dpx::set_error(int code, const char* msg) { return fail(code, "%s", msg); }

// Bracket assignment of IntegrateLayersTogether (Amplitude.cpp:1184-1217);
// where two brackets claim one q, the later layer wins.
void dpx::q_brackets(int grid_size, double qmax, int nq, const double* Q, int* layer_of_q) {
    const int L = grid_size / 2;
    const double step = 2 * qmax / grid_size;
    for (int k = 0; k < nq; ++k) layer_of_q[k] = -1;
    if (nq == 0) return;
    int tmp = 0;
    while (Q[0] > (tmp + 1) * step) tmp++;
    // qb = the length of the prefix of Q at or below layer * step: it only
    // grows with the layer (for any Q), so each layer's scan continues the last
    int qb = 0;
    for (int layer = tmp; layer < L; ++layer) {
        while (qb < nq && Q[qb] <= layer * step) qb++;
        if (qb >= nq) continue;
        int qe = qb + 1;
        if (qe == nq) qe--;
        while (qe + 1 != nq && Q[qe] <= (layer + 1) * step) qe++;
        if (qe + 1 != nq) qe--;
        for (int k = qb; k <= qe; ++k) layer_of_q[k] = layer;
    }
}

namespace {
using dpx::q_brackets;

}  // namespace

int dpxh::grid_from_voxels(int64_t voxels, int thDivs, int phDivs, double stepSize, int* grid_size, double* qmax) {
    if (thDivs != 3 || phDivs != 6) return fail(DPX_ERR_ARG, "only thDivs=3, phDivs=6 grids exist");
    for (int lp = 4; lp < 4096; ++lp) {
        const int64_t P = 6 * (int64_t)lp * (lp + 1) * (lp + 1) + 1;
        if (P == voxels) {
            *grid_size = 2 * (lp - 3);
            *qmax = stepSize * (lp - 3);
            return DPX_OK;
        }
        if (P > voxels) break;
    }
    return fail(DPX_ERR_ARG, "voxels=%lld is not a Jacobian sphere grid size", (long long)voxels);
}

extern "C" {

const char* dpx_last_error(void) { return g_err.c_str(); }
int dpx_version(void) { return 1; }

int dpx_ctx_create(int device, dpx_ctx* out) {
    if (!out) return fail(DPX_ERR_ARG, "out is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(DPX_ERR_NODEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
    }
    if (device < 0 || device >= n) return fail(DPX_ERR_ARG, "device %d out of range", device);
    DPX_CUDA(cudaSetDevice(device));
    dpx_ctx c = new dpx_ctx_s();
    c->device = device;
    e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreate");
    }
    c->stream = c->own;
    *out = c;
    return DPX_OK;
}

}  // extern "C"

namespace dpxh {
void ctx_retain(dpx_ctx ctx) { ++ctx->refs; }

// Frees the context once the caller has destroyed it and no grid uses it.
void ctx_release(dpx_ctx ctx) {
    if (--ctx->refs > 0) return;
    set_device(ctx);
    cudaStreamSynchronize(ctx->stream);
    for (DevBuf* b : {&ctx->atoms, &ctx->table, &ctx->ions, &ctx->models, &ctx->groups, &ctx->plan, &ctx->partial,
                      &ctx->result, &ctx->dirs, &ctx->debye, &ctx->harmonic, &ctx->dirsort, &ctx->direct})
        b->release();
    for (cudaEvent_t e : ctx->tev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->aev)
        if (e) cudaEventDestroy(e);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
}
}  // namespace dpxh

extern "C" {

int dpx_ctx_destroy(dpx_ctx ctx) {
    if (!ctx) return DPX_OK;
    if (ctx->closed) return fail(DPX_ERR_ARG, "context destroyed twice");
    ctx->closed = true;
    ctx_release(ctx);
    return DPX_OK;
}

int dpx_ctx_set_stream(dpx_ctx ctx, void* stream) {
    if (!ctx) return fail(DPX_ERR_ARG, "ctx is NULL");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
    return DPX_OK;
}

void* dpx_ctx_get_stream(dpx_ctx ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int dpx_ctx_synchronize(dpx_ctx ctx) {
    if (!ctx) return fail(DPX_ERR_ARG, "ctx is NULL");
    DPX_CUDA(cudaStreamSynchronize(ctx->stream));
    return DPX_OK;
}

int dpx_ctx_set_fill_shape(dpx_ctx ctx, int cpt, int threads) {
    if (!ctx) return fail(DPX_ERR_ARG, "ctx is NULL");
    for (int k = 0; k < kFillShapes; ++k)
        if (cpt > 0 && kFillShape[k][0] == cpt && kFillShape[k][1] == threads) {
            ctx->fill_cpt = cpt;
            ctx->fill_threads = threads;
            ctx->fill_poly = 0;
            return DPX_OK;
        }
    return fail(DPX_ERR_ARG, "unsupported fill shape %d cells x %d threads", cpt, threads);
}

int dpx_ctx_set_fill_poly(dpx_ctx ctx, int poly_columns) {
    if (!ctx) return fail(DPX_ERR_ARG, "ctx is NULL");
    for (int k = 0; k < kFillShapes; ++k)
        if (kFillShape[k][0] == ctx->fill_cpt && kFillShape[k][1] == ctx->fill_threads &&
            kFillShape[k][3] == poly_columns) {
            ctx->fill_poly = poly_columns;
            return DPX_OK;
        }
    return fail(DPX_ERR_ARG, "no %d x %d fill with %d FMA-pipe columns", ctx->fill_cpt, ctx->fill_threads,
                poly_columns);
}

int dpx_ctx_set_convergence(dpx_ctx ctx, int rule, int64_t samples_per_step) {
    if (!ctx) return fail(DPX_ERR_ARG, "ctx is NULL");
    if (rule != DPX_CONV_CPU && rule != DPX_CONV_GPU) return fail(DPX_ERR_ARG, "unknown convergence rule %d", rule);
    if (rule == DPX_CONV_GPU && (samples_per_step < 128 || samples_per_step % 128 != 0))
        return fail(DPX_ERR_ARG, "samples_per_step must be a positive multiple of 128");
    ctx->conv_rule = rule;
    if (rule == DPX_CONV_GPU) ctx->conv_samples = samples_per_step;
    return DPX_OK;
}

int dpx_ctx_set_timing(dpx_ctx ctx, int on) {
    if (!ctx) return fail(DPX_ERR_ARG, "ctx is NULL");
    ctx->timing = on != 0;
    ctx->tev_used = 0;
    ctx->aev_used = false;
    return DPX_OK;
}

int dpx_ctx_average_kernel_ms(dpx_ctx ctx, double* ms) {
    if (!ctx || !ms) return fail(DPX_ERR_ARG, "NULL argument");
    *ms = 0.0;
    if (!ctx->aev_used) return DPX_OK;
    if (int rc = set_device(ctx)) return rc;
    DPX_CUDA(cudaEventSynchronize(ctx->aev[1]));
    float f = 0.f;
    DPX_CUDA(cudaEventElapsedTime(&f, ctx->aev[0], ctx->aev[1]));
    *ms = f;
    return DPX_OK;
}

int dpx_ctx_stage_times(dpx_ctx ctx, double* out) {
    if (!ctx || !out) return fail(DPX_ERR_ARG, "NULL argument");
    for (int k = 0; k < 5; ++k) out[k] = 0.0;
    if (ctx->tev_used == 0) return DPX_OK;
    if (int rc = set_device(ctx)) return rc;
    DPX_CUDA(cudaEventSynchronize(ctx->tev[7]));
    float ms = 0.f;
    DPX_CUDA(cudaEventElapsedTime(&ms, ctx->tev[0], ctx->tev[1]));
    out[0] = ms;
    if (ctx->tev_used == 8) {
        DPX_CUDA(cudaEventElapsedTime(&ms, ctx->tev[2], ctx->tev[3]));
        out[0] += ms;
    }
    DPX_CUDA(cudaEventElapsedTime(&ms, ctx->tev[4], ctx->tev[5]));
    out[1] = ms;
    DPX_CUDA(cudaEventElapsedTime(&ms, ctx->tev[6], ctx->tev[7]));
    out[2] = ms;
    out[3] = ctx->stage_points;
    out[4] = ctx->stage_k;
    return DPX_OK;
}

int dpx_ctx_set_fill_method(dpx_ctx ctx, int method) {
    if (!ctx) return fail(DPX_ERR_ARG, "ctx is NULL");
    if (method != DPX_FILL_DIRECT && method != DPX_FILL_HARMONIC) return fail(DPX_ERR_ARG, "unknown fill method %d", method);
    ctx->fill_method = method;
    return DPX_OK;
}

int dpx_ctx_get_fill_method(dpx_ctx ctx) { return ctx ? ctx->fill_method : DPX_ERR_ARG; }

int dpx_set_average_shape(int directions_per_thread) {
    if (dpx::set_average_dpt(directions_per_thread) != 0)
        return fail(DPX_ERR_ARG, "directions per thread must be 1 or 2, got %d", directions_per_thread);
    return DPX_OK;
}

int dpx_set_moments_kernel(int kind) {
    if (kind != DPX_MOMENTS_TCGEN05 && kind != DPX_MOMENTS_MMA_SYNC && kind != DPX_MOMENTS_MMA_F16)
        return fail(DPX_ERR_ARG, "unknown moments kernel %d", kind);
    dpx::set_moments_kernel(kind);
    return DPX_OK;
}

int dpx_get_moments_kernel(void) { return dpx::moments_kernel(); }

int dpx_take_device_faults(unsigned* flags) {
    if (!flags) return fail(DPX_ERR_ARG, "NULL argument");
    *flags = 0;
    DPX_CUDA(dpx::harmonic_take_faults(flags));
    return DPX_OK;
}

int dpx_ctx_set_fill_schedule(dpx_ctx ctx, int persistent) {
    if (!ctx) return fail(DPX_ERR_ARG, "ctx is NULL");
    ctx->fill_persistent = persistent != 0;
    return DPX_OK;
}

int dpx_ctx_get_fill_shape(dpx_ctx ctx, int* shape) {
    if (!ctx || !shape) return fail(DPX_ERR_ARG, "NULL argument");
    shape[0] = ctx->fill_cpt;
    shape[1] = ctx->fill_threads;
    shape[2] = ctx->fill_persistent;
    shape[3] = ctx->fill_poly;
    return DPX_OK;
}

int dpx_fill_shapes(int* shapes) {
    if (shapes)
        for (int k = 0; k < kFillShapes; ++k)
            for (int j = 0; j < 4; ++j) shapes[4 * k + j] = kFillShape[k][j];
    return kFillShapes;
}

int64_t dpx_grid_cells(int grid_size) {
    if (grid_size < 2) return -1;
    return dpx::make_geom(grid_size, 1.0).P;
}

int64_t dpx_grid_bytes(int grid_size, int precision) {
    const int64_t p = dpx_grid_cells(grid_size);
    return p < 0 ? -1 : p * (int64_t)cell_bytes(precision);
}

int dpx_grid_create(dpx_ctx ctx, int grid_size, double qmax, int precision, dpx_grid* out) {
    if (!ctx || !out) return fail(DPX_ERR_ARG, "NULL argument");
    if (grid_size < 2 || (grid_size & 1)) return fail(DPX_ERR_ARG, "grid_size must be even and >= 2");
    if (!(qmax > 0)) return fail(DPX_ERR_ARG, "qmax must be positive");
    if (precision != DPX_FP32 && precision != DPX_FP64) return fail(DPX_ERR_ARG, "bad precision");
    if (int rc = set_device(ctx)) return rc;
    dpx_grid g = new dpx_grid_s();
    g->ctx = ctx;
    g->grid_size = grid_size;
    g->qmax = qmax;
    g->precision = precision;
    g->g = dpx::make_geom(grid_size, qmax);
    cudaError_t e = cudaMalloc(&g->cells, (size_t)g->g.P * cell_bytes(precision));
    if (e != cudaSuccess) {
        delete g;
        return cuda_fail(e, "cudaMalloc(grid)");
    }
    e = cudaMemsetAsync(g->cells, 0, (size_t)g->g.P * cell_bytes(precision), ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(g->cells);
        delete g;
        return cuda_fail(e, "cudaMemset(grid)");
    }
    ctx->refs++;
    *out = g;
    return DPX_OK;
}

int dpx_grid_destroy(dpx_grid g) {
    if (!g) return DPX_OK;
    set_device(g->ctx);
    cudaStreamSynchronize(g->ctx->stream);
    cudaFree(g->cells);
    dpx_ctx ctx = g->ctx;
    delete g;
    ctx_release(ctx);
    return DPX_OK;
}

void* dpx_grid_device_ptr(dpx_grid g) {
    if (!g) return nullptr;
    g->splines_current = false;  // the caller may write through it
    return g->cells;
}

int dpx_grid_info(dpx_grid g, int* grid_size, double* qmax, int* precision, int64_t* cells) {
    if (!g) return fail(DPX_ERR_ARG, "grid is NULL");
    if (grid_size) *grid_size = g->grid_size;
    if (qmax) *qmax = g->qmax;
    if (precision) *precision = g->precision;
    if (cells) *cells = g->g.P;
    return DPX_OK;
}

}  // extern "C"

namespace dpxh {

// Validate one leaf description; returns DPX_OK or an argument error.
int check_pdb(const dpx_pdb_desc& d) {
    if (d.n_atoms <= 0 || !d.atoms) return fail(DPX_ERR_ARG, "no atoms");
    if (d.n_atoms > INT_MAX) return fail(DPX_ERR_ARG, "too many atoms (%lld)", (long long)d.n_atoms);
    if (d.n_ions <= 0 || d.n_ions > 256 || !d.atoms_per_ion || (!d.aff && (!d.coeffs || !d.ion_rads)))
        return fail(DPX_ERR_ARG, "bad ion description");
    if (d.aff && d.aff_n <= 0) return fail(DPX_ERR_ARG, "aff_n must be positive with a tabulated aff");
    int64_t tot = 0;
    for (int u = 0; u < d.n_ions; ++u) {
        if (d.atoms_per_ion[u] < 0) return fail(DPX_ERR_ARG, "negative atoms_per_ion");
        tot += d.atoms_per_ion[u];
    }
    if (tot != d.n_atoms)
        return fail(DPX_ERR_ARG, "atoms_per_ion sums to %lld, n_atoms=%lld", (long long)tot, (long long)d.n_atoms);
    return DPX_OK;
}

int ctx_harmonic_streams(dpx_ctx ctx, HarmStreams& S) {
    if (ctx->timing)
        for (cudaEvent_t& e : ctx->tev)
            if (!e) DPX_CUDA(cudaEventCreate(&e));
    S = HarmStreams{};
    S.st = ctx->stream;
    S.tev = ctx->timing ? ctx->tev : nullptr;
    return DPX_OK;
}

void ctx_stage_record(dpx_ctx ctx, const HarmPlan& p) {
    if (!ctx->timing) return;
    ctx->tev_used = 6;  // moments (both point sets in one launch), synthesis, the whole fill
    ctx->stage_points = p.stage_points;
    ctx->stage_k = p.stage_k;
}

// Batched fill with an explicit FP32 launch shape; ev0/ev1 (optional) bracket
// the FP32 fill launch on the context's stream.
int fill_batch_impl(int n, const dpx_grid* grids, const dpx_pdb_desc* pdbs, int cpt, int threads, int poly,
                    bool persistent, cudaEvent_t ev0, cudaEvent_t ev1) {
    if (n <= 0 || !grids || !pdbs) return fail(DPX_ERR_ARG, "empty batch");
    dpx_ctx ctx = grids[0] ? grids[0]->ctx : nullptr;
    for (int j = 0; j < n; ++j) {
        if (!grids[j] || grids[j]->ctx != ctx) return fail(DPX_ERR_ARG, "every grid of a batch needs the same context");
        if (int rc = check_pdb(pdbs[j])) return rc;
        if (int rc = check_leaf_grid(pdbs[j], grids[j]->g)) return rc;
        for (int k = 0; k < j; ++k)
            if (grids[k] == grids[j]) return fail(DPX_ERR_ARG, "a grid appears twice in one batch");
    }
    if (int rc = set_device(ctx)) return rc;
    cudaStream_t s = ctx->stream;
    for (int j = 0; j < n; ++j) grids[j]->splines_current = false;

    // the harmonic method plans the FP32 leaves it takes (host work and
    // synchronizations), the rest are staged for the direct sum
    std::vector<char> harm(n, 0);
    std::vector<HarmPlan> plans(n);
    struct Release {
        std::vector<HarmPlan>& p;
        ~Release() {
            for (HarmPlan& x : p) harmonic_plan_release(x);
        }
    } release{plans};
    if (ctx->fill_method == DPX_FILL_HARMONIC)
        for (int j = 0; j < n; ++j) {
            if (grids[j]->precision != DPX_FP32) continue;
            const int rc = harmonic_plan(s, pdbs[j], grids[j]->g, plans[j]);
            if (rc < 0) return rc;
            harm[j] = rc == DPX_OK;
        }
    // host staging of every direct leaf, then the FP32 job table and the tile counter
    std::vector<char>& h = ctx->host_stage;
    h.clear();
    std::vector<LeafTables> lt(n);
    for (int j = 0; j < n; ++j) {
        if (harm[j]) continue;
        const bool fp32 = grids[j]->precision == DPX_FP32;
        stage_leaf(h, pdbs[j], grids[j]->g, fp32, fp32 ? cpt : dpx::kFill64Cells, lt[j]);
    }
    const size_t jobs_off = al16(h.size());
    const size_t counter_off = al16(jobs_off + (size_t)n * sizeof(dpx::FillJob));
    h.resize(counter_off + 64, 0);
    DPX_CUDA(ctx->atoms.reserve(h.size()));
    const char* dbase = (const char*)ctx->atoms.p;
    DPX_CUDA(cudaMemcpyAsync(ctx->atoms.p, h.data(), jobs_off, cudaMemcpyHostToDevice, s));
    if (ev0) DPX_CUDA(cudaEventRecord(ev0, s));
    size_t scratch = 0;
    for (int j = 0; j < n; ++j)
        if (harm[j]) scratch = std::max(scratch, plans[j].scratch_bytes);
    if (scratch) {
        if (cudaError_t e = ctx->harmonic.reserve(scratch)) {
            cudaGetLastError();
            return fail(DPX_ERR_OOM, "harmonic fill needs %zu bytes of scratch (%s)", scratch, cudaGetErrorString(e));
        }
        HarmStreams S;
        if (int rc = ctx_harmonic_streams(ctx, S)) return rc;
        for (int j = 0; j < n; ++j) {
            if (!harm[j]) continue;
            if (int rc = harmonic_launch(S, plans[j], ctx->harmonic.p, reinterpret_cast<float4*>(grids[j]->cells)))
                return rc;
            ctx_stage_record(ctx, plans[j]);
        }
    }
    std::vector<dpx::FillJob> jobs;
    int64_t tiles = 0;
    for (int j = 0; j < n; ++j) {
        if (grids[j]->precision != DPX_FP32 || harm[j]) continue;
        jobs.push_back(make_job(pdbs[j], lt[j], dbase, grids[j]->g, grids[j]->cells, tiles));
        tiles += (lt[j].items + threads - 1) / threads;
    }
    if (!jobs.empty()) {
        std::memcpy(h.data() + jobs_off, jobs.data(), jobs.size() * sizeof(dpx::FillJob));
        DPX_CUDA(cudaMemcpyAsync(static_cast<char*>(ctx->atoms.p) + jobs_off, h.data() + jobs_off, counter_off - jobs_off,
                                 cudaMemcpyHostToDevice, s));
    }
    bool boxes = false;
    for (const dpx::FillJob& J : jobs) boxes |= J.n_boxes > 0;
    cudaError_t e = dpx::launch_fill_f32_batch(s, (const dpx::FillJob*)(dbase + jobs_off), (int)jobs.size(), tiles,
                                               (unsigned long long*)(dbase + counter_off), cpt, threads, poly,
                                               persistent, boxes);
    if (e != cudaSuccess) return cuda_fail(e, "amplitude fill launch");
    if (ev1) DPX_CUDA(cudaEventRecord(ev1, s));
    for (int j = 0; j < n; ++j) {  // the plain FP64 path: one launch per leaf
        if (grids[j]->precision != DPX_FP64) continue;
        e = launch_leaf_f64(s, pdbs[j], lt[j], dbase, grids[j]->g, grids[j]->cells);
        if (e != cudaSuccess) return cuda_fail(e, "amplitude fill launch");
    }
    // the staging buffer is reused by the next call: wait for the copy and the kernels
    DPX_CUDA(cudaStreamSynchronize(s));
    for (int j = 0; j < n; ++j) grids[j]->splines_current = harm[j] != 0;  // the synthesis wrote them
    return DPX_OK;
}

}  // namespace dpxh

extern "C" {

int dpx_grid_fill_pdb_batch(int n, const dpx_grid* grids, const dpx_pdb_desc* pdbs) {
    if (n <= 0 || !grids || !grids[0]) return fail(DPX_ERR_ARG, "empty batch");
    const dpx_ctx ctx = grids[0]->ctx;
    return fill_batch_impl(n, grids, pdbs, ctx->fill_cpt, ctx->fill_threads, ctx->fill_poly, ctx->fill_persistent,
                           nullptr, nullptr);
}

int dpx_autotune_fill(int n, const dpx_grid* grids, const dpx_pdb_desc* pdbs, int repeats, int* best,
                      float* times_ms) {
    if (n <= 0 || !grids || !grids[0] || !pdbs) return fail(DPX_ERR_ARG, "empty batch");
    if (repeats <= 0) return fail(DPX_ERR_ARG, "repeats must be positive");
    const dpx_ctx ctx = grids[0]->ctx;
    if (int rc = set_device(ctx)) return rc;
    cudaEvent_t e0, e1;
    DPX_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(DPX_ERR_CUDA, "cudaEventCreate");
    }
    int rc = DPX_OK, bi = -1;
    float bt = 0.f;
    const int method0 = ctx->fill_method;
    for (int k = 0; k < kFillShapes && !rc; ++k) {
        float tot = 0.f;
        const bool harmonic = kFillShape[k][0] == 0;
        ctx->fill_method = harmonic ? DPX_FILL_HARMONIC : DPX_FILL_DIRECT;
        for (int r = 0; r <= repeats && !rc; ++r) {  // r = 0 warms up
            rc = harmonic ? fill_batch_impl(n, grids, pdbs, ctx->fill_cpt, ctx->fill_threads, ctx->fill_poly,
                                            ctx->fill_persistent, e0, e1)
                          : fill_batch_impl(n, grids, pdbs, kFillShape[k][0], kFillShape[k][1], kFillShape[k][3],
                                            kFillShape[k][2] != 0, e0, e1);
            float ms = 0.f;
            if (!rc && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = fail(DPX_ERR_CUDA, "event timing");
            if (r > 0) tot += ms;
        }
        const float avg = tot / repeats;
        if (times_ms) times_ms[k] = avg;
        if (!rc && (bi < 0 || avg < bt)) {
            bi = k;
            bt = avg;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->fill_method = method0;
    if (rc) return rc;
    if (kFillShape[bi][0] == 0) {
        ctx->fill_method = DPX_FILL_HARMONIC;
    } else {
        ctx->fill_method = DPX_FILL_DIRECT;
        ctx->fill_cpt = kFillShape[bi][0];
        ctx->fill_threads = kFillShape[bi][1];
        ctx->fill_persistent = kFillShape[bi][2] != 0;
        ctx->fill_poly = kFillShape[bi][3];
    }
    if (best)
        for (int j = 0; j < 4; ++j) best[j] = kFillShape[bi][j];
    // leave the grids filled with the chosen shape: shapes with FMA-pipe
    // columns differ from the SFU ones in the last bits
    if (bi != kFillShapes - 1)
        return fill_batch_impl(n, grids, pdbs, ctx->fill_cpt, ctx->fill_threads, ctx->fill_poly, ctx->fill_persistent,
                               nullptr, nullptr);
    return DPX_OK;
}

int dpx_grid_fill_pdb(dpx_grid g, int64_t n_atoms, const float* atoms, int atoms_on_device, int n_ions,
                      const int* atoms_per_ion, const double* coeffs, const double* ion_rads, int flags,
                      double solvent_ed, double c1, double scale, const double* center) {
    if (!g) return fail(DPX_ERR_ARG, "grid is NULL");
    dpx_pdb_desc d{n_atoms, atoms, atoms_on_device, n_ions, atoms_per_ion, coeffs, ion_rads, flags,
                   solvent_ed, c1, scale, center, 0, nullptr, 0.0};
    return dpx_grid_fill_pdb_batch(1, &g, &d);
}

int dpx_grid_compute_splines(dpx_grid g) {
    if (!g) return fail(DPX_ERR_ARG, "grid is NULL");
    if (g->splines_current) return DPX_OK;  // written with the values, the same bits
    if (int rc = set_device(g->ctx)) return rc;
    cudaError_t e = g->precision == DPX_FP64 ? dpx::launch_splines_f64(g->ctx->stream, g->g, (double4_32a*)g->cells)
                                             : dpx::launch_splines_f32(g->ctx->stream, g->g, (float4*)g->cells);
    if (e != cudaSuccess) return cuda_fail(e, "spline launch");
    g->splines_current = true;
    return DPX_OK;
}

int dpx_grid_read(dpx_grid g, double* values, double* coeffs) {
    if (!g) return fail(DPX_ERR_ARG, "grid is NULL");
    dpx_ctx ctx = g->ctx;
    if (int rc = set_device(ctx)) return rc;
    const size_t n = (size_t)g->g.P * 2 * sizeof(double);
    DPX_CUDA(ctx->partial.reserve(n));
    for (int which = 0; which < 2; ++which) {
        double* dst = which ? coeffs : values;
        if (!dst) continue;
        cudaError_t e;
        if (g->precision == DPX_FP64)
            e = which ? dpx::launch_pack_ders_f64(ctx->stream, (double4_32a*)g->cells, g->g.P, (double*)ctx->partial.p)
                      : dpx::launch_pack_values_f64(ctx->stream, (double4_32a*)g->cells, g->g.P, (double*)ctx->partial.p);
        else
            e = which ? dpx::launch_pack_ders_f32(ctx->stream, (float4*)g->cells, g->g.P, (double*)ctx->partial.p)
                      : dpx::launch_pack_values_f32(ctx->stream, (float4*)g->cells, g->g.P, (double*)ctx->partial.p);
        if (e != cudaSuccess) return cuda_fail(e, "pack launch");
        DPX_CUDA(cudaMemcpyAsync(dst, ctx->partial.p, n, cudaMemcpyDeviceToHost, ctx->stream));
        DPX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return DPX_OK;
}

int dpx_grid_write(dpx_grid g, const double* values, const double* coeffs) {
    if (!g || !values) return fail(DPX_ERR_ARG, "NULL argument");
    g->splines_current = false;
    dpx_ctx ctx = g->ctx;
    if (int rc = set_device(ctx)) return rc;
    const size_t n = (size_t)g->g.P * 2 * sizeof(double);
    DPX_CUDA(ctx->partial.reserve(2 * n));
    double* dv = (double*)ctx->partial.p;
    double* dd = coeffs ? dv + 2 * g->g.P : nullptr;
    DPX_CUDA(cudaMemcpyAsync(dv, values, n, cudaMemcpyHostToDevice, ctx->stream));
    if (coeffs) DPX_CUDA(cudaMemcpyAsync(dd, coeffs, n, cudaMemcpyHostToDevice, ctx->stream));
    cudaError_t e = g->precision == DPX_FP64 ? dpx::launch_unpack_f64(ctx->stream, dv, dd, g->g.P, (double4_32a*)g->cells)
                                             : dpx::launch_unpack_f32(ctx->stream, dv, dd, g->g.P, (float4*)g->cells);
    if (e != cudaSuccess) return cuda_fail(e, "unpack launch");
    DPX_CUDA(cudaStreamSynchronize(ctx->stream));
    return DPX_OK;
}

}  // extern "C"

namespace dpxh {
// Model structs and docked rotation groups (ManualSymmetry translationsPerOrientation
// grouped by identical Euler triples, first-appearance order); group tables are
// staged for ctx->groups, model structs point into it.
void make_brackets(const dpx::Geom& G, int grid_size, double qmax, int nq, const double* Q, Brackets& b) {
    std::vector<int> layer_of_q(nq);
    dpx::q_brackets(grid_size, qmax, nq, Q, layer_of_q.data());
    b = Brackets{};
    // the q of each layer in ascending layer order, each layer's in index order
    // (a stable counting pass)
    std::vector<int> start(G.L + 1, 0);
    for (int k = 0; k < nq; ++k)
        if (layer_of_q[k] >= 0 && layer_of_q[k] < G.L) start[layer_of_q[k] + 1]++;
    for (int l = 0; l < G.L; ++l) start[l + 1] += start[l];
    std::vector<int> order(start[G.L]);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int k = 0; k < nq; ++k)
        if (layer_of_q[k] >= 0 && layer_of_q[k] < G.L) order[fill[layer_of_q[k]]++] = k;
    for (int l = 0; l < G.L; ++l) {
        const int cnt = start[l + 1] - start[l];
        if (!cnt) continue;
        for (int j = start[l]; j < start[l + 1]; ++j) {
            b.q.push_back(Q[order[j]]);
            b.qidx.push_back(order[j]);
        }
        b.layer.push_back(l);
        b.off.push_back((int)b.q.size());
        b.max_q = std::max(b.max_q, cnt);
    }
}

namespace {
struct TripleHash {
    size_t operator()(const std::array<double, 3>& a) const {
        uint64_t h = 1469598103934665603ull;
        for (double v : a) {
            uint64_t b;
            std::memcpy(&b, &v, sizeof b);
            h = (h ^ b) * 1099511628211ull;
        }
        return (size_t)h;
    }
};

// Translations t_m = t_0 + m d (m = 0..M-1) to 1e-9 nm on every axis, in the
// order given: the group's phase sum then has a closed form (the FP32 path uses it).
bool arithmetic_progression(const std::vector<double>& T, size_t first, size_t M, double d[3]) {
    if (M < 3) return false;
    const double* t0 = &T[3 * first];
    const double* tl = &T[3 * (first + M - 1)];
    for (int a = 0; a < 3; ++a) d[a] = (tl[a] - t0[a]) / double(M - 1);
    for (size_t m = 1; m + 1 < M; ++m)
        for (int a = 0; a < 3; ++a)
            if (std::fabs(T[3 * (first + m) + a] - (t0[a] + double(m) * d[a])) > 1e-9) return false;
    return true;
}
}  // namespace

int build_models(int n_models, const void* const* cells, const double* rot, const double* tr, const int* n_copies,
                 const double* copy_rot, const double* copy_tr, const double* sym_scale, ModelTables& t) {
    std::vector<dpx::ModelDev>& md = t.md;
    std::vector<char>& gstage = t.gstage;
    md.assign(n_models, dpx::ModelDev{});
    std::vector<double> gR, gT, gS, gW;
    std::vector<float> gRf;
    std::vector<int> gOff, gA;
    std::vector<int> model_group_base(n_models), model_toff_base(n_models), model_gidx_base(n_models);
    int copy_base = 0;
    for (int m = 0; m < n_models; ++m) {
        dpx::ModelDev& M = md[m];
        M.grid = cells[m];
        euler(rot ? rot[3 * m] : 0, rot ? rot[3 * m + 1] : 0, rot ? rot[3 * m + 2] : 0, M.R);
        for (int k = 0; k < 3; ++k) M.tr[k] = tr ? tr[3 * m + k] : 0.0;
        const int nc = n_copies ? n_copies[m] : 0;
        M.sym_scale = sym_scale ? sym_scale[m] : 1.0;
        M.plain = (M.R[0] == 1.0 && M.R[4] == 1.0 && M.R[8] == 1.0 && M.R[1] == 0.0 && M.R[2] == 0.0 &&
                   M.R[3] == 0.0 && M.R[5] == 0.0 && M.R[6] == 0.0 && M.R[7] == 0.0 && M.tr[0] == 0.0 &&
                   M.tr[1] == 0.0 && M.tr[2] == 0.0);
        for (int k = 0; k < 9; ++k) M.Rf[k] = (float)M.R[k];
        for (int i = 0; i < 3; ++i) M.w[i] = M.R[3 * i] * M.tr[0] + M.R[3 * i + 1] * M.tr[1] + M.R[3 * i + 2] * M.tr[2];
        model_group_base[m] = (int)gOff.size();
        model_gidx_base[m] = (int)gA.size();
        // group copies by identical Euler triples, first-appearance order
        // (ManualSymmetry translationsPerOrientation, Symmetries.cpp:670-695)
        std::unordered_map<std::array<double, 3>, int, TripleHash> where;
        std::vector<std::vector<int>> members;
        for (int c = 0; c < nc; ++c) {
            const double* r = copy_rot + 3 * (copy_base + c);
            const std::array<double, 3> key{r[0], r[1], r[2]};
            auto f = where.find(key);
            if (f == where.end()) {
                where.emplace(key, (int)members.size());
                members.push_back({c});
            } else {
                members[f->second].push_back(c);
            }
        }
        M.n_groups = (int)members.size();
        model_toff_base[m] = (int)(gT.size() / 3);
        for (size_t gi = 0; gi < members.size(); ++gi) {
            double R[9];
            const double* r = copy_rot + 3 * (copy_base + members[gi][0]);
            euler(r[0], r[1], r[2], R);
            gR.insert(gR.end(), R, R + 9);
            // FP32 average: C = R_copy R_leaf (the sample's leaf frame is C^T n) and
            // w = C t_leaf (its leaf phase is q n.w, kept in FP64)
            double Cm[9], w[3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    Cm[3 * i + j] = R[3 * i] * M.R[j] + R[3 * i + 1] * M.R[3 + j] + R[3 * i + 2] * M.R[6 + j];
            for (int i = 0; i < 3; ++i) w[i] = Cm[3 * i] * M.tr[0] + Cm[3 * i + 1] * M.tr[1] + Cm[3 * i + 2] * M.tr[2];
            for (int k = 0; k < 9; ++k) gRf.push_back((float)Cm[k]);
            gW.insert(gW.end(), w, w + 3);
            const size_t first = gT.size() / 3;
            gOff.push_back((int)first - model_toff_base[m]);
            for (int c : members[gi]) {
                const double* tt = copy_tr + 3 * (copy_base + c);
                gT.insert(gT.end(), tt, tt + 3);
            }
            double d[3] = {0, 0, 0};
            const bool ap = arithmetic_progression(gT, first, members[gi].size(), d);
            gS.insert(gS.end(), d, d + 3);
            gA.push_back(ap ? (int)members[gi].size() : 0);
        }
        gOff.push_back((int)(gT.size() / 3) - model_toff_base[m]);
        copy_base += nc;
    }
    // device layout of the group tables: [R][T][step] (doubles) [off][ap] (ints)
    // [R][T][step][w] (doubles) [C] (floats) [off][ap] (ints); the ints start at
    // bytesD + bytesF
    const size_t bytesR = gR.size() * sizeof(double), bytesT = gT.size() * sizeof(double),
                 bytesS = gS.size() * sizeof(double), bytesW = gW.size() * sizeof(double),
                 bytesF = gRf.size() * sizeof(float), bytesO0 = gOff.size() * sizeof(int),
                 bytesA = gA.size() * sizeof(int);
    const size_t bytesD = bytesR + bytesT + bytesS + bytesW;
    const size_t bytesO = bytesF + bytesO0;  // everything before the ap ints, after the doubles
    gstage.assign(bytesD + bytesO + bytesA, 0);
    char* h = gstage.data();
    if (bytesR) std::memcpy(h, gR.data(), bytesR);
    if (bytesT) std::memcpy(h + bytesR, gT.data(), bytesT);
    if (bytesS) std::memcpy(h + bytesR + bytesT, gS.data(), bytesS);
    if (bytesW) std::memcpy(h + bytesR + bytesT + bytesS, gW.data(), bytesW);
    if (bytesF) std::memcpy(h + bytesD, gRf.data(), bytesF);
    if (bytesO0) std::memcpy(h + bytesD + bytesF, gOff.data(), bytesO0);
    if (bytesA) std::memcpy(h + bytesD + bytesO, gA.data(), bytesA);
    t.oR.assign(n_models, 0);
    t.oT.assign(n_models, 0);
    t.oO.assign(n_models, 0);
    t.oS.assign(n_models, 0);
    t.oA.assign(n_models, 0);
    t.oW.assign(n_models, 0);
    t.oF.assign(n_models, 0);
    int groups_seen = 0;
    for (int m = 0; m < n_models; ++m) {
        t.oR[m] = 9 * sizeof(double) * (size_t)groups_seen;
        t.oS[m] = bytesR + bytesT + 3 * sizeof(double) * (size_t)groups_seen;
        t.oW[m] = bytesR + bytesT + bytesS + 3 * sizeof(double) * (size_t)groups_seen;
        t.oF[m] = bytesD + 9 * sizeof(float) * (size_t)groups_seen;
        t.oO[m] = bytesD + bytesF + sizeof(int) * (size_t)model_group_base[m];
        t.oA[m] = bytesD + bytesO + sizeof(int) * (size_t)model_gidx_base[m];
        t.oT[m] = bytesR + 3 * sizeof(double) * (size_t)model_toff_base[m];
        groups_seen += md[m].n_groups;
    }
    return DPX_OK;
}

void place_models(ModelTables& t, char* dbase) {
    for (size_t m = 0; m < t.md.size(); ++m) {
        t.md[m].group_R = reinterpret_cast<const double*>(dbase + t.oR[m]);
        t.md[m].group_off = reinterpret_cast<const int*>(dbase + t.oO[m]);
        t.md[m].trans = reinterpret_cast<const double*>(dbase + t.oT[m]);
        t.md[m].group_step = reinterpret_cast<const double*>(dbase + t.oS[m]);
        t.md[m].group_ap = reinterpret_cast<const int*>(dbase + t.oA[m]);
        t.md[m].group_w = reinterpret_cast<const double*>(dbase + t.oW[m]);
        t.md[m].group_Cf = reinterpret_cast<const float*>(dbase + t.oF[m]);
    }
}

int prepare_models(dpx_ctx ctx, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                   const int* n_copies, const double* copy_rot, const double* copy_tr, const double* sym_scale,
                   std::vector<dpx::ModelDev>& md, std::vector<char>& gstage) {
    std::vector<const void*> cells(n_models);
    for (int m = 0; m < n_models; ++m) cells[m] = grids[m]->cells;
    ModelTables t;
    if (int rc = build_models(n_models, cells.data(), rot, tr, n_copies, copy_rot, copy_tr, sym_scale, t)) return rc;
    DPX_CUDA(ctx->groups.reserve(t.gstage.size() + 64));
    place_models(t, (char*)ctx->groups.p);
    md.swap(t.md);
    gstage.swap(t.gstage);
    return DPX_OK;
}

}  // namespace dpxh

extern "C" {

int dpx_orientation_average(dpx_ctx ctx, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                            const int* n_copies, const double* copy_rot, const double* copy_tr,
                            const double* sym_scale, int nq, const double* Q, const double* dirs, int dirs_on_device,
                            int64_t dir_layer_stride, int64_t n_samples, double eps, double* res) {
    if (!ctx || n_models <= 0 || !grids || nq <= 0 || !Q || !dirs || !res)
        return fail(DPX_ERR_ARG, "NULL or empty argument");
    if (n_samples <= 0) return fail(DPX_ERR_ARG, "n_samples must be positive");
    const int grid_size = grids[0]->grid_size;
    const double qmax = grids[0]->qmax;
    const int prec = grids[0]->precision;
    for (int m = 0; m < n_models; ++m)
        if (!grids[m] || grids[m]->grid_size != grid_size || grids[m]->qmax != qmax || grids[m]->precision != prec)
            return fail(DPX_ERR_ARG, "all models must share grid_size, qmax and precision");
    for (int k = 1; k < nq; ++k)
        if (!(Q[k] >= Q[k - 1])) return fail(DPX_ERR_ARG, "Q must be ascending");
    if (Q[0] < 0) return fail(DPX_ERR_ARG, "negative q");
    const Geom& G = grids[0]->g;
    if (Q[nq - 1] > G.L * G.step * (1.0 + 1e-12))
        return fail(DPX_ERR_ARG, "q=%g beyond the grid's qmax=%g", Q[nq - 1], G.L * G.step);
    if (int rc = set_device(ctx)) return rc;
    cudaStream_t s = ctx->stream;

    std::vector<dpx::ModelDev> md;
    std::vector<char> gstage;
    if (int rc = prepare_models(ctx, n_models, grids, rot, tr, n_copies, copy_rot, copy_tr, sym_scale, md, gstage))
        return rc;


    // brackets
    Brackets B;
    make_brackets(G, grid_size, qmax, nq, Q, B);
    const std::vector<int>&br_layer = B.layer, &br_off = B.off, &br_qidx = B.qidx;
    const std::vector<double>& br_q = B.q;
    const int max_q = B.max_q;
    const int nbr = (int)br_layer.size();
    dpx::AvgPlan plan{};
    plan.n_brackets = nbr;
    plan.max_q = max_q;
    plan.n_samples = n_samples;
    const bool gpu_rule = eps > 0.0 && ctx->conv_rule == DPX_CONV_GPU;
    plan.chunk = eps > 0.0 && !gpu_rule ? 100 : 128;
    plan.chunk_off = eps > 0.0 && !gpu_rule ? 99 : 0;
    plan.n_chunks = (n_samples + plan.chunk_off + plan.chunk - 1) / plan.chunk;
    plan.conv_group = gpu_rule ? (int)(ctx->conv_samples / 128) : 0;
    plan.dir_stride = dir_layer_stride;
    plan.need_dir = 0;
    for (const auto& M : md)
        if (!M.plain || M.n_groups > 0) plan.need_dir = 1;
    plan.one_leaf = (n_models == 1 && md[0].n_groups == 0) ? 1 : 0;
    const size_t pb = br_layer.size() * sizeof(int) + br_off.size() * sizeof(int) + br_qidx.size() * sizeof(int) +
                      br_q.size() * sizeof(double) + 64;
    DPX_CUDA(ctx->plan.reserve(pb + md.size() * sizeof(dpx::ModelDev) + 64));
    std::vector<char> stage(pb + md.size() * sizeof(dpx::ModelDev) + 64);
    size_t o = 0;
    auto put = [&](const void* src, size_t n) -> size_t {
        size_t at = (o + 15) & ~size_t(15);
        if (n) std::memcpy(stage.data() + at, src, n);
        o = at + n;
        return at;
    };
    const size_t oQ = put(br_q.data(), br_q.size() * sizeof(double));
    const size_t oL = put(br_layer.data(), br_layer.size() * sizeof(int));
    const size_t oO = put(br_off.data(), br_off.size() * sizeof(int));
    const size_t oI = put(br_qidx.data(), br_qidx.size() * sizeof(int));
    const size_t oM = put(md.data(), md.size() * sizeof(dpx::ModelDev));
    char* pbase = (char*)ctx->plan.p;
    plan.br_q = (const double*)(pbase + oQ);
    plan.br_layer = (const int*)(pbase + oL);
    plan.br_q_off = (const int*)(pbase + oO);
    plan.br_qidx = (const int*)(pbase + oI);
    const dpx::ModelDev* d_models = (const dpx::ModelDev*)(pbase + oM);

    // directions
    if (dirs_on_device) {
        plan.dirs = dirs;
    } else {
        const int64_t nd = (dir_layer_stride ? (int64_t)(G.L - 1) * dir_layer_stride : 0) + n_samples;
        DPX_CUDA(ctx->dirs.reserve((size_t)nd * 2 * sizeof(double)));
        DPX_CUDA(cudaMemcpyAsync(ctx->dirs.p, dirs, (size_t)nd * 2 * sizeof(double), cudaMemcpyHostToDevice, s));
        plan.dirs = (const double*)ctx->dirs.p;
    }
    const size_t part = ((size_t)nbr * plan.n_chunks + (size_t)nbr * 5) * max_q * sizeof(double) + 64;
    DPX_CUDA(ctx->partial.reserve(part));
    plan.partial = (double*)ctx->partial.p;
    // eps = 0 with one direction set: the samples in angular order (the same mean)
    if (eps == 0.0 && dir_layer_stride == 0) {
        DPX_CUDA(ctx->dirsort.reserve(dpx::dir_sort_bytes(n_samples)));
        plan.sort_scratch = (int*)ctx->dirsort.p;
    }
    DPX_CUDA(ctx->result.reserve((size_t)nq * sizeof(double)));
    DPX_CUDA(cudaMemcpyAsync(ctx->plan.p, stage.data(), o, cudaMemcpyHostToDevice, s));
    DPX_CUDA(cudaMemcpyAsync(ctx->groups.p, gstage.data(), gstage.size(), cudaMemcpyHostToDevice, s));
    DPX_CUDA(cudaMemsetAsync(ctx->result.p, 0, (size_t)nq * sizeof(double), s));

    if (ctx->timing)
        for (cudaEvent_t& ev : ctx->aev)
            if (!ev) DPX_CUDA(cudaEventCreate(&ev));
    cudaError_t e = dpx::launch_average(s, prec == DPX_FP64, G, n_models, d_models, plan,
                                        ctx->timing ? ctx->aev : nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "average launch");
    ctx->aev_used = ctx->timing;
    e = dpx::launch_finalize(s, plan, eps, (double*)ctx->result.p);
    if (e != cudaSuccess) return cuda_fail(e, "finalize launch");
    DPX_CUDA(cudaMemcpyAsync(res, ctx->result.p, (size_t)nq * sizeof(double), cudaMemcpyDeviceToHost, s));

    // q == 0: |sum of leaves at the origin|^2 (Amplitude.cpp:1176-1182)
    std::vector<double> origin(4 * n_models, 0.0);
    for (int m = 0; m < n_models; ++m) {
        if (prec == DPX_FP64) {
            DPX_CUDA(cudaMemcpyAsync(&origin[4 * m], grids[m]->cells, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        } else {
            float2 v;
            DPX_CUDA(cudaMemcpyAsync(&v, grids[m]->cells, sizeof(float2), cudaMemcpyDeviceToHost, s));
            DPX_CUDA(cudaStreamSynchronize(s));
            origin[4 * m] = v.x;
            origin[4 * m + 1] = v.y;
        }
    }
    DPX_CUDA(cudaStreamSynchronize(s));
    if (Q[0] == 0.0) {
        double ar = 0, ai = 0;
        for (int m = 0; m < n_models; ++m) {
            double w = 1.0;
            if (md[m].n_groups > 0) w = (n_copies ? n_copies[m] : 0) * md[m].sym_scale;
            ar += w * origin[4 * m];
            ai += w * origin[4 * m + 1];
        }
        res[0] = ar * ar + ai * ai;
    }
    return DPX_OK;
}

int dpx_vegas_intensity(dpx_ctx ctx, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                        const int* n_copies, const double* copy_rot, const double* copy_tr, const double* sym_scale,
                        int nq, const double* Q, uint64_t seed, int points_per_iter, int64_t max_points, double eps,
                        double* res) {
    if (!ctx || n_models <= 0 || !grids || nq <= 0 || !Q || !res) return fail(DPX_ERR_ARG, "NULL or empty argument");
    if (points_per_iter <= 0 || points_per_iter % 1024)
        return fail(DPX_ERR_ARG, "points_per_iter must be a positive multiple of 1024 (32 x 32 bins)");
    if (max_points <= 0) return fail(DPX_ERR_ARG, "max_points must be positive");
    const int grid_size = grids[0]->grid_size;
    const double qmax = grids[0]->qmax;
    const int prec = grids[0]->precision;
    for (int m = 0; m < n_models; ++m)
        if (!grids[m] || grids[m]->grid_size != grid_size || grids[m]->qmax != qmax || grids[m]->precision != prec)
            return fail(DPX_ERR_ARG, "all models must share grid_size, qmax and precision");
    for (int k = 1; k < nq; ++k)
        if (!(Q[k] >= Q[k - 1])) return fail(DPX_ERR_ARG, "Q must be ascending");
    if (!(Q[0] >= 0)) return fail(DPX_ERR_ARG, "negative q");
    const Geom& G = grids[0]->g;
    if (Q[nq - 1] > G.L * G.step * (1.0 + 1e-12))
        return fail(DPX_ERR_ARG, "q=%g beyond the grid's qmax=%g", Q[nq - 1], G.L * G.step);
    if (int rc = set_device(ctx)) return rc;
    cudaStream_t s = ctx->stream;

    std::vector<dpx::ModelDev> md;
    std::vector<char> gstage;
    if (int rc = prepare_models(ctx, n_models, grids, rot, tr, n_copies, copy_rot, copy_tr, sym_scale, md, gstage))
        return rc;
    int need_dir = 0;
    for (const auto& M : md)
        if (!M.plain || M.n_groups > 0) need_dir = 1;

    // brackets of the hybrid path (GPUHybridCalc.cu:363-375), q = 0 included
    struct Br { int q0, m; };
    std::vector<Br> brs;
    int max_m = 1;
    for (int qInd = 0, lower = 0; qInd < nq;) {
        while (Q[qInd] > double(lower + 1) * G.step) lower++;
        int qEnd;
        for (qEnd = qInd + 1; qEnd < nq; qEnd++)
            if (Q[qEnd] > double(lower + 1) * G.step) break;
        qEnd--;
        brs.push_back({qInd, qEnd - qInd + 1});
        max_m = std::max(max_m, qEnd - qInd + 1);
        qInd = qEnd + 1;
        lower++;
    }
    const int n_iter = (int)((max_points + points_per_iter - 1) / points_per_iter);

    // device layout in ctx->plan: [models][bounds 66][q nq][qidx nq][done nbr][hist n_iter x max_m]; I in ctx->partial
    std::vector<int> qidx(nq);
    for (int k = 0; k < nq; ++k) qidx[k] = k;
    std::vector<double> bounds(2 * 32 + 2);
    for (int i = 0; i <= 32; ++i) bounds[i] = double(i) / 32;
    for (int i = 0; i <= 32; ++i) bounds[33 + i] = double(i) / 32;
    std::vector<char> stage;
    size_t o = 0;
    auto put = [&](const void* src, size_t n) -> size_t {
        size_t at = (o + 31) & ~size_t(31);
        stage.resize(at + n);
        if (n) std::memcpy(stage.data() + at, src, n);
        o = at + n;
        return at;
    };
    const size_t oM = put(md.data(), md.size() * sizeof(dpx::ModelDev));
    const size_t oB = put(bounds.data(), bounds.size() * sizeof(double));
    const size_t oQ = put(Q, (size_t)nq * sizeof(double));
    const size_t oI = put(qidx.data(), qidx.size() * sizeof(int));
    std::vector<int> zeros(brs.size(), 0);
    const size_t oD = put(zeros.data(), zeros.size() * sizeof(int));
    const size_t oH = (o + 31) & ~size_t(31);
    const size_t total = oH + (size_t)n_iter * max_m * sizeof(double);
    DPX_CUDA(ctx->plan.reserve(total));
    DPX_CUDA(ctx->partial.reserve((size_t)points_per_iter * max_m * sizeof(double)));
    DPX_CUDA(ctx->result.reserve((size_t)nq * sizeof(double)));
    char* base = (char*)ctx->plan.p;
    DPX_CUDA(cudaMemcpyAsync(base, stage.data(), o, cudaMemcpyHostToDevice, s));
    DPX_CUDA(cudaMemcpyAsync(ctx->groups.p, gstage.data(), gstage.size(), cudaMemcpyHostToDevice, s));
    const dpx::ModelDev* d_models = (const dpx::ModelDev*)(base + oM);
    double* d_bounds = (double*)(base + oB);
    const double* d_q = (const double*)(base + oQ);
    const int* d_qidx = (const int*)(base + oI);
    int* d_done = (int*)(base + oD);
    double* d_hist = (double*)(base + oH);
    double* d_I = (double*)ctx->partial.p;
    double* d_res = (double*)ctx->result.p;
    for (size_t b = 0; b < brs.size(); ++b) {
        for (int it = 0; it < n_iter; ++it) {
            const uint64_t key = (uint64_t(b) << 32) | uint64_t(it);
            cudaError_t e = dpx::launch_vegas_points(s, prec == DPX_FP64, G, n_models, d_models, need_dir,
                                                     d_q + brs[b].q0, brs[b].m, points_per_iter, seed, key, d_bounds,
                                                     d_done + b, d_I);
            if (e == cudaSuccess)
                e = dpx::launch_vegas_update(s, d_bounds, d_I, brs[b].m, points_per_iter, it, eps, d_hist, d_done + b,
                                             d_res, d_qidx + brs[b].q0);
            if (e != cudaSuccess) return cuda_fail(e, "VEGAS launch");
        }
    }
    DPX_CUDA(cudaMemcpyAsync(res, d_res, (size_t)nq * sizeof(double), cudaMemcpyDeviceToHost, s));
    DPX_CUDA(cudaStreamSynchronize(s));
    return DPX_OK;
}

int dpx_grid_assemble(dpx_grid dst, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                      const int* n_copies, const double* copy_rot, const double* copy_tr, const double* sym_scale,
                      const double* lattice, double scale) {
    if (!dst || n_models <= 0 || !grids) return fail(DPX_ERR_ARG, "NULL or empty argument");
    for (int m = 0; m < n_models; ++m) {
        if (!grids[m] || grids[m]->grid_size != dst->grid_size || grids[m]->qmax != dst->qmax ||
            grids[m]->precision != dst->precision)
            return fail(DPX_ERR_ARG, "source grids must share the destination's grid_size, qmax and precision");
        if (grids[m] == dst) return fail(DPX_ERR_ARG, "the destination cannot also be a source");
    }
    dst->splines_current = false;
    dpx_ctx ctx = dst->ctx;
    if (int rc = set_device(ctx)) return rc;
    cudaStream_t s = ctx->stream;
    std::vector<dpx::ModelDev> md;
    std::vector<char> gstage;
    if (int rc = prepare_models(ctx, n_models, grids, rot, tr, n_copies, copy_rot, copy_tr, sym_scale, md, gstage))
        return rc;
    DPX_CUDA(ctx->models.reserve(md.size() * sizeof(dpx::ModelDev)));
    DPX_CUDA(cudaMemcpyAsync(ctx->models.p, md.data(), md.size() * sizeof(dpx::ModelDev), cudaMemcpyHostToDevice, s));
    DPX_CUDA(cudaMemcpyAsync(ctx->groups.p, gstage.data(), gstage.size(), cudaMemcpyHostToDevice, s));
    cudaError_t e = dpx::launch_assemble(s, dst->precision == DPX_FP64, dst->g, n_models,
                                         (const dpx::ModelDev*)ctx->models.p, lattice, scale, dst->cells);
    if (e != cudaSuccess) return cuda_fail(e, "assembly launch");
    DPX_CUDA(cudaStreamSynchronize(s));  // the staged host vectors go out of scope
    return DPX_OK;
}

int dpx_gk_intensity(dpx_ctx ctx, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                     const int* n_copies, const double* copy_rot, const double* copy_tr, const double* sym_scale,
                     int nq, const double* Q, double eps, int64_t max_depth, double* res) {
    if (!ctx || n_models <= 0 || !grids || nq <= 0 || !Q || !res) return fail(DPX_ERR_ARG, "NULL or empty argument");
    const int grid_size = grids[0]->grid_size;
    const double qmax = grids[0]->qmax;
    const int prec = grids[0]->precision;
    for (int m = 0; m < n_models; ++m)
        if (!grids[m] || grids[m]->grid_size != grid_size || grids[m]->qmax != qmax || grids[m]->precision != prec)
            return fail(DPX_ERR_ARG, "all models must share grid_size, qmax and precision");
    for (int k = 0; k < nq; ++k)
        if (!(Q[k] >= 0)) return fail(DPX_ERR_ARG, "negative q");
    const Geom& G = grids[0]->g;
    for (int k = 0; k < nq; ++k)
        if (Q[k] > G.L * G.step * (1.0 + 1e-12)) return fail(DPX_ERR_ARG, "q=%g beyond the grid's qmax", Q[k]);
    if (int rc = set_device(ctx)) return rc;
    cudaStream_t s = ctx->stream;
    std::vector<dpx::ModelDev> md;
    std::vector<char> gstage;
    if (int rc = prepare_models(ctx, n_models, grids, rot, tr, n_copies, copy_rot, copy_tr, sym_scale, md, gstage))
        return rc;
    DPX_CUDA(ctx->models.reserve(md.size() * sizeof(dpx::ModelDev)));
    DPX_CUDA(cudaMemcpyAsync(ctx->models.p, md.data(), md.size() * sizeof(dpx::ModelDev), cudaMemcpyHostToDevice, s));
    DPX_CUDA(cudaMemcpyAsync(ctx->groups.p, gstage.data(), gstage.size(), cudaMemcpyHostToDevice, s));
    const dpx::ModelDev* d_models = (const dpx::ModelDev*)ctx->models.p;

    // the 7/15 rule (the standard published Gauss-Kronrod pair)
    static const double x15[15] = {
        -0.9914553711208126392068547, -0.9491079123427585245261897, -0.8648644233597690727897128,
        -0.7415311855993944398638648, -0.5860872354676911302941448, -0.4058451513773971669066064,
        -0.2077849550078984676006894, 0.0, 0.2077849550078984676006894, 0.4058451513773971669066064,
        0.5860872354676911302941448, 0.7415311855993944398638648, 0.8648644233597690727897128,
        0.9491079123427585245261897, 0.9914553711208126392068547};
    static const double w15[15] = {
        0.0229353220105292249637320, 0.0630920926299785532907007, 0.1047900103222501838398763,
        0.1406532597155259187451896, 0.1690047266392679028265834, 0.1903505780647854099132564,
        0.2044329400752988924141620, 0.2094821410847278280129992, 0.2044329400752988924141620,
        0.1903505780647854099132564, 0.1690047266392679028265834, 0.1406532597155259187451896,
        0.1047900103222501838398763, 0.0630920926299785532907007, 0.0229353220105292249637320};
    static const double w7[7] = {0.1294849661688696932706114, 0.2797053914892766679014678,
                                 0.3818300505051189449503698, 0.4179591836734693877551020,
                                 0.3818300505051189449503698, 0.2797053914892766679014678,
                                 0.1294849661688696932706114};
    struct ThetaIv { int q; double tmin, tmax; int64_t depth; };
    struct Node { double st, ct, sum; };
    struct PhiIv { int node; double pmin, pmax; int64_t depth; };
    const int64_t kMaxTasks = 1 << 24;
    std::vector<double> acc(nq, 0.0);
    std::vector<ThetaIv> thetas;
    for (int k = 0; k < nq; ++k)
        if (Q[k] > 0.0) thetas.push_back({k, 0.0, kPi / 2, max_depth - 1});  // GaussKron2DSphereRecurs
    std::vector<dpx::GKTask> tasks;
    std::vector<double2> kg;
    while (!thetas.empty()) {
        std::vector<Node> nodes(thetas.size() * 15);
        std::vector<PhiIv> phis;
        for (size_t t = 0; t < thetas.size(); ++t) {
            const double ba2 = (thetas[t].tmax - thetas[t].tmin) * 0.5, apb2 = (thetas[t].tmax + thetas[t].tmin) * 0.5;
            for (int i = 0; i < 15; ++i) {
                const double tv = apb2 + ba2 * x15[i];
                nodes[t * 15 + i] = {std::sin(tv), std::cos(tv), 0.0};
                phis.push_back({(int)(t * 15 + i), 0.0, 2.0 * kPi, thetas[t].depth});
            }
        }
        while (!phis.empty()) {
            if ((int64_t)phis.size() > kMaxTasks)
                return fail(DPX_ERR_ARG, "Gauss-Kronrod needs more than %lld phi intervals at once; raise eps or "
                                         "lower max_depth", (long long)kMaxTasks);
            tasks.resize(phis.size());
            for (size_t p = 0; p < phis.size(); ++p) {
                const Node& nd = nodes[phis[p].node];
                tasks[p] = {Q[thetas[phis[p].node / 15].q], nd.st, nd.ct, phis[p].pmin, phis[p].pmax};
            }
            kg.resize(phis.size());
            DPX_CUDA(ctx->plan.reserve(tasks.size() * sizeof(dpx::GKTask)));
            DPX_CUDA(ctx->partial.reserve(kg.size() * sizeof(double2)));
            DPX_CUDA(cudaMemcpyAsync(ctx->plan.p, tasks.data(), tasks.size() * sizeof(dpx::GKTask),
                                     cudaMemcpyHostToDevice, s));
            cudaError_t e = dpx::launch_gk_phi(s, prec == DPX_FP64, G, n_models, d_models,
                                               (const dpx::GKTask*)ctx->plan.p, (int)tasks.size(),
                                               (double2*)ctx->partial.p);
            if (e != cudaSuccess) return cuda_fail(e, "Gauss-Kronrod launch");
            DPX_CUDA(cudaMemcpyAsync(kg.data(), ctx->partial.p, kg.size() * sizeof(double2), cudaMemcpyDeviceToHost,
                                     s));
            DPX_CUDA(cudaStreamSynchronize(s));
            std::vector<PhiIv> next;
            for (size_t p = 0; p < phis.size(); ++p) {
                const double kv = kg[p].x, gv = kg[p].y;
                // GaussLegPhi acceptance (Amplitude.cpp:1460)
                if (phis[p].depth < 0 || std::fabs(1.0 - gv / kv) <= eps || gv == kv) {
                    nodes[phis[p].node].sum += kv;
                } else {
                    const double mid = (phis[p].pmin + phis[p].pmax) * 0.5;
                    next.push_back({phis[p].node, phis[p].pmin, mid, phis[p].depth - 1});
                    next.push_back({phis[p].node, mid, phis[p].pmax, phis[p].depth - 1});
                }
            }
            phis.swap(next);
        }
        std::vector<ThetaIv> next_t;
        for (size_t t = 0; t < thetas.size(); ++t) {
            const double ba2 = (thetas[t].tmax - thetas[t].tmin) * 0.5;
            double kv = 0, gv = 0;
            for (int i = 0; i < 15; ++i) {
                const Node& nd = nodes[t * 15 + i];
                kv += nd.sum * w15[i] * ba2 * nd.st;
                if (i % 2 == 1) gv += nd.sum * w7[i / 2] * ba2 * nd.st;
            }
            // GaussLegTheta acceptance (Amplitude.cpp:1434)
            if (thetas[t].depth < 0 || std::fabs(1.0 - gv / kv) <= eps || gv == kv) {
                acc[thetas[t].q] += kv;
            } else {
                const double mid = (thetas[t].tmax + thetas[t].tmin) / 2.0;
                next_t.push_back({thetas[t].q, thetas[t].tmin, mid, thetas[t].depth - 1});
                next_t.push_back({thetas[t].q, mid, thetas[t].tmax, thetas[t].depth - 1});
            }
        }
        thetas.swap(next_t);
    }
    // q == 0: |sum of models at the origin|^2 (CalculateIntensity, Amplitude.cpp:1477-1482)
    double o_r = 0, o_i = 0;
    for (int m = 0; m < n_models; ++m) {
        double v[2] = {0, 0};
        if (prec == DPX_FP64) {
            DPX_CUDA(cudaMemcpy(v, grids[m]->cells, 2 * sizeof(double), cudaMemcpyDeviceToHost));
        } else {
            float f[2];
            DPX_CUDA(cudaMemcpy(f, grids[m]->cells, 2 * sizeof(float), cudaMemcpyDeviceToHost));
            v[0] = f[0];
            v[1] = f[1];
        }
        const double w = md[m].n_groups > 0 ? (n_copies ? n_copies[m] : 0) * md[m].sym_scale : 1.0;
        o_r += w * v[0];
        o_i += w * v[1];
    }
    for (int k = 0; k < nq; ++k) res[k] = (Q[k] > 0.0) ? acc[k] / (2.0 * kPi) : o_r * o_r + o_i * o_i;
    return DPX_OK;
}

int dpx_measure_sfu_peak(dpx_ctx ctx, double* ops_per_s) {
    if (!ctx || !ops_per_s) return fail(DPX_ERR_ARG, "NULL argument");
    if (int rc = set_device(ctx)) return rc;
    int dev = 0, sms = 0;
    DPX_CUDA(cudaGetDevice(&dev));
    DPX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, iters = 4096;
    cudaStream_t s = ctx->stream;
    DPX_CUDA(ctx->result.reserve(64));
    cudaEvent_t e0, e1;
    DPX_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(DPX_ERR_CUDA, "cudaEventCreate");
    }
    cudaError_t e = dpx::launch_sfu_probe(s, blocks, 64, (float*)ctx->result.p);  // warm-up
    float best = 0.f;
    for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
        cudaEventRecord(e0, s);
        e = dpx::launch_sfu_probe(s, blocks, iters, (float*)ctx->result.p);
        cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && (best == 0.f || ms < best)) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(e, "SFU probe");
    *ops_per_s = double(blocks) * 256.0 * iters * 8 * 2 / (best * 1e-3);
    return DPX_OK;
}

int dpx_measure_tcgen05_issue(dpx_ctx ctx, double* cycles_per_mma) {
    if (!ctx || !cycles_per_mma) return fail(DPX_ERR_ARG, "NULL argument");
    if (int rc = set_device(ctx)) return rc;
    DPX_CUDA(ctx->result.reserve(64));
    char* d = static_cast<char*>(ctx->result.p);
    DPX_CUDA(cudaMemsetAsync(d, 0, 64, ctx->stream));
    DPX_CUDA(dpx::launch_tc_issue_probe(ctx->stream, reinterpret_cast<long long*>(d), reinterpret_cast<int*>(d + 16)));
    long long c[2] = {0, 0};
    int st = 0;
    DPX_CUDA(cudaMemcpyAsync(c, d, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
    DPX_CUDA(cudaMemcpyAsync(&st, d + 16, sizeof st, cudaMemcpyDeviceToHost, ctx->stream));
    DPX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (st) return fail(DPX_ERR_CUDA, "tcgen05 issue probe: a wait ran past its limit");
    for (int k = 0; k < 2; ++k) cycles_per_mma[k] = (double)c[k] / dpx::tc_issue_probe_mmas();
    return DPX_OK;
}

int dpx_measure_pipe_peaks(dpx_ctx ctx, double* flops_per_s) {
    if (!ctx || !flops_per_s) return fail(DPX_ERR_ARG, "NULL argument");
    if (int rc = set_device(ctx)) return rc;
    int dev = 0, sms = 0;
    DPX_CUDA(cudaGetDevice(&dev));
    DPX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s = ctx->stream;
    DPX_CUDA(ctx->result.reserve(64));
    cudaEvent_t e0, e1;
    DPX_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(DPX_ERR_CUDA, "cudaEventCreate");
    }
    cudaError_t e = cudaSuccess;
    const int blocks = sms * 8;
    for (int kind = 0; kind < 4 && e == cudaSuccess; ++kind) {
        const int iters = kind >= 2 ? 2048 : 8192;
        e = dpx::launch_pipe_probe(s, kind, blocks, 64, (float*)ctx->result.p);  // warm-up
        float best = 0.f;
        for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
            cudaEventRecord(e0, s);
            e = dpx::launch_pipe_probe(s, kind, blocks, iters, (float*)ctx->result.p);
            cudaEventRecord(e1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e == cudaSuccess && (best == 0.f || ms < best)) best = ms;
        }
        const double threads = double(blocks) * 256.0;
        const double flops = kind == 0 ? threads * iters * 8 * 2
                             : kind == 1 ? threads * iters * 8 * 4
                             : kind == 2 ? threads / 32.0 * iters * 4 * 2048.0
                                         : threads / 32.0 * iters * 4 * 4096.0;
        if (e == cudaSuccess) flops_per_s[kind] = flops / (best * 1e-3);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(e, "pipe probe");
    return DPX_OK;
}

int dpx_mc_directions(uint32_t seed, int64_t D, double* theta_phi) {
    if (D < 0 || (D > 0 && !theta_phi)) return fail(DPX_ERR_ARG, "bad direction buffer");
    std::mt19937 rng;
    rng.seed(seed);
    std::uniform_real_distribution<double> u(0.0, 2.0);
    for (int64_t i = 0; i < D; ++i) {
        const double u2 = u(rng);
        const double v2 = u(rng);
        theta_phi[2 * i + 1] = u2 * kPi;
        theta_phi[2 * i] = std::acos(v2 - 1.0);
    }
    return DPX_OK;
}

int dpx_layer_seeds(uint32_t master, int nq, int n_layers, uint32_t* seeds) {
    if (!seeds || nq < 0 || n_layers < 0) return fail(DPX_ERR_ARG, "bad arguments");
    std::mt19937 gen;
    std::uniform_int_distribution<unsigned int> draw(0, UINT_MAX);
    gen.seed(master);
    for (int i = 0; i < nq; ++i) (void)draw(gen);
    for (int i = 0; i <= n_layers; ++i) seeds[i] = draw(gen);
    return DPX_OK;
}

int dpx_q_brackets(int grid_size, double qmax, int nq, const double* Q, int* layer_of_q) {
    if (grid_size < 2 || nq < 0 || (nq > 0 && (!Q || !layer_of_q))) return fail(DPX_ERR_ARG, "bad arguments");
    q_brackets(grid_size, qmax, nq, Q, layer_of_q);
    return DPX_OK;
}

int dpx_make_globule(int64_t n_atoms, double radius_nm, uint64_t seed, float* xyz, int* elem) {
    if (n_atoms <= 0 || !(radius_nm > 0) || !xyz || !elem) return fail(DPX_ERR_ARG, "bad arguments");
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U01(0.0, 1.0);
    const double step = 0.15, min_d = 0.1, cell = 0.2;
    const double R = radius_nm;
    const int nc = (int)std::ceil(2 * R / cell) + 2;
    auto key = [&](double x, double y, double z) -> int64_t {
        int64_t ix = (int64_t)std::floor((x + R) / cell) + 1, iy = (int64_t)std::floor((y + R) / cell) + 1,
                iz = (int64_t)std::floor((z + R) / cell) + 1;
        return (ix * nc + iy) * nc + iz;
    };
    std::unordered_map<int64_t, std::vector<int64_t>> cells;
    cells.reserve((size_t)n_atoms * 2);
    auto free_at = [&](double x, double y, double z) -> bool {
        const int64_t ix = (int64_t)std::floor((x + R) / cell) + 1, iy = (int64_t)std::floor((y + R) / cell) + 1,
                      iz = (int64_t)std::floor((z + R) / cell) + 1;
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    auto it = cells.find(((ix + dx) * nc + (iy + dy)) * nc + (iz + dz));
                    if (it == cells.end()) continue;
                    for (int64_t j : it->second) {
                        const double ex = xyz[3 * j] - x, ey = xyz[3 * j + 1] - y, ez = xyz[3 * j + 2] - z;
                        if (ex * ex + ey * ey + ez * ez < min_d * min_d) return false;
                    }
                }
        return true;
    };
    double px = 0, py = 0, pz = 0;
    for (int64_t i = 0; i < n_atoms; ++i) {
        double x = px, y = py, z = pz;
        if (i > 0) {
            bool placed = false;
            for (int attempt = 0; attempt < 64 && !placed; ++attempt) {
                const double ct = 2 * U01(rng) - 1, ph = 2 * kPi * U01(rng), st = std::sqrt(1 - ct * ct);
                x = px + step * st * std::cos(ph);
                y = py + step * st * std::sin(ph);
                z = pz + step * ct;
                if (x * x + y * y + z * z > R * R) continue;
                placed = free_at(x, y, z);
            }
            if (!placed) {
                // dead end: restart the chain at a random free point inside the sphere
                for (int attempt = 0; attempt < 100000; ++attempt) {
                    x = (2 * U01(rng) - 1) * R;
                    y = (2 * U01(rng) - 1) * R;
                    z = (2 * U01(rng) - 1) * R;
                    if (x * x + y * y + z * z <= R * R && free_at(x, y, z)) { placed = true; break; }
                }
                if (!placed) return fail(DPX_ERR_ARG, "globule of radius %g nm cannot hold %lld atoms", R,
                                         (long long)n_atoms);
            }
        }
        xyz[3 * i] = (float)x;
        xyz[3 * i + 1] = (float)y;
        xyz[3 * i + 2] = (float)z;
        cells[key(x, y, z)].push_back(i);
        px = x; py = y; pz = z;
        const double r = U01(rng);
        elem[i] = r < 0.63 ? 0 : (r < 0.80 ? 1 : (r < 0.99 ? 2 : 3));
    }
    return DPX_OK;
}

namespace {
// The body of both grid-amplitude drop-ins: form factors from coefficients
// (coeffs, ionRads) or tabulated (affs, nq).
int pdb_grid_amplitude(uint64_t voxels, int thDivs, int phDivs, double stepSize, double* outData,
                       const float* atomLocations, int64_t numAtoms, int numUniqueIons, const int* atomsPerIon,
                       const float* coeffs, const float* ionRads, const float* affs, int nq, int bitCombination,
                       float solventED, float c1, const float* solCOM, const int* solDims, int64_t nSol,
                       double voxStep, const float* outSolCOM, const int* outSolDims, int64_t nOutSol,
                       double outerSolED, double scale, int precision, int* pStop);
}  // namespace

int dpx_pdb_jacobian_grid_amplitude(uint64_t voxels, int thDivs, int phDivs, double stepSize, double* outData,
                                    const float* atomLocations, int64_t numAtoms, int numUniqueIons,
                                    const int* atomsPerIon, const float* coeffs, const float* ionRads,
                                    int bitCombination, float solventED, float c1, const float* solCOM,
                                    const int* solDims, int64_t nSol, double voxStep, const float* outSolCOM,
                                    const int* outSolDims, int64_t nOutSol, double outerSolED, double scale,
                                    int precision, int* pStop) {
    if (!coeffs) return fail(DPX_ERR_ARG, "NULL coefficients");
    return pdb_grid_amplitude(voxels, thDivs, phDivs, stepSize, outData, atomLocations, numAtoms, numUniqueIons,
                              atomsPerIon, coeffs, ionRads, nullptr, 0, bitCombination, solventED, c1, solCOM,
                              solDims, nSol, voxStep, outSolCOM, outSolDims, nOutSol, outerSolED, scale, precision,
                              pStop);
}

int dpx_pdb_jacobian_grid_amplitude_aff(uint64_t voxels, int thDivs, int phDivs, double stepSize, double* outData,
                                        const float* atomLocations, int64_t numAtoms, int numUniqueIons,
                                        const int* atomsPerIon, const float* affs, int nq, int bitCombination,
                                        float solventED, const float* solCOM, const int* solDims, int64_t nSol,
                                        double voxStep, const float* outSolCOM, const int* outSolDims,
                                        int64_t nOutSol, double outerSolED, double scale, int precision, int* pStop) {
    if (!affs || nq <= 0) return fail(DPX_ERR_ARG, "NULL form-factor table");
    return pdb_grid_amplitude(voxels, thDivs, phDivs, stepSize, outData, atomLocations, numAtoms, numUniqueIons,
                              atomsPerIon, nullptr, nullptr, affs, nq, bitCombination, solventED, 1.0f, solCOM,
                              solDims, nSol, voxStep, outSolCOM, outSolDims, nOutSol, outerSolED, scale, precision,
                              pStop);
}

}  // extern "C"

namespace {
int pdb_grid_amplitude(uint64_t voxels, int thDivs, int phDivs, double stepSize, double* outData,
                       const float* atomLocations, int64_t numAtoms, int numUniqueIons, const int* atomsPerIon,
                       const float* coeffs, const float* ionRads, const float* affs, int nq, int bitCombination,
                       float solventED, float c1, const float* solCOM, const int* solDims, int64_t nSol,
                       double voxStep, const float* outSolCOM, const int* outSolDims, int64_t nOutSol,
                       double outerSolED, double scale, int precision, int* pStop) {
    if (!outData || !atomLocations) return fail(DPX_ERR_ARG, "NULL buffer");
    if (numUniqueIons <= 0 || numUniqueIons > 256 || !atomsPerIon) return fail(DPX_ERR_ARG, "bad ion description");
    if ((nSol > 0 && (!solCOM || !solDims)) || (nOutSol > 0 && (!outSolCOM || !outSolDims)))
        return fail(DPX_ERR_ARG, "NULL voxel arrays");
    // voxel boxes as PDBJacobianGridAmplitudeCalculation applies them
    // (PDBAmplitudeCUDA.cu:363-389): excluded volume at -solvED when the
    // CALC_VOXELIZED_SOLVENT bit (1 << 3) is set, the outer layer at
    // outerSolED - solvED, each only with more than four boxes
    std::vector<float> boxes;
    auto add = [&](const float* com, const int* dims, int64_t n, double w) {
        for (int64_t b = 0; b < n; ++b) {
            const float rec[8] = {com[4 * b], com[4 * b + 1], com[4 * b + 2], (float)w,
                                  (float)voxStep * (float)dims[4 * b], (float)voxStep * (float)dims[4 * b + 1],
                                  (float)voxStep * (float)dims[4 * b + 2], 0.f};
            boxes.insert(boxes.end(), rec, rec + 8);
        }
    };
    if (solventED != 0.0f && (bitCombination & (1 << 3)) && nSol > 4) add(solCOM, solDims, nSol, -solventED);
    if (outerSolED != 0.0 && nOutSol > 4) add(outSolCOM, outSolDims, nOutSol, outerSolED - solventED);
    int grid_size;
    double qmax;
    if (int rc = grid_from_voxels((int64_t)voxels, thDivs, phDivs, stepSize, &grid_size, &qmax)) return rc;
    if (pStop && *pStop) return fail(DPX_ERR_STOPPED, "stopped");
    int dev = 0;
    cudaGetDevice(&dev);
    dpx_ctx ctx;
    if (int rc = dpx_ctx_create(dev, &ctx)) return rc;
    dpx_grid g;
    int rc = dpx_grid_create(ctx, grid_size, qmax, precision, &g);
    if (rc) { dpx_ctx_destroy(ctx); return rc; }
    std::vector<double> cd(coeffs ? 9 * numUniqueIons : 0), rd(coeffs ? numUniqueIons : 0);
    for (size_t k = 0; k < cd.size(); ++k) cd[k] = coeffs[k];
    for (size_t k = 0; k < rd.size(); ++k) rd[k] = ionRads ? ionRads[k] : 0.0;
    dpx_pdb_desc d{numAtoms, atomLocations, 0, numUniqueIons, atomsPerIon, coeffs ? cd.data() : nullptr,
                   coeffs ? rd.data() : nullptr, bitCombination & 3, solventED, c1, scale, nullptr,
                   (int64_t)boxes.size() / 8, boxes.empty() ? nullptr : boxes.data(), voxStep, affs, nq};
    rc = dpx_grid_fill_pdb_batch(1, &g, &d);
    if (!rc && pStop && *pStop) rc = fail(DPX_ERR_STOPPED, "stopped");
    if (!rc) rc = dpx_grid_read(g, outData, nullptr);
    dpx_grid_destroy(g);
    dpx_ctx_destroy(ctx);
    return rc;
}
}  // namespace

extern "C" {

int dpx_calc_mcoa_jacob_sphr(int64_t voxels, int thDivs, int phDivs, double stepSz, const double* inAmp,
                             const double* inD, const double* qs, double* intensities, int qPoints, int64_t maxIters,
                             double convergence, const double* dirs, int64_t dir_layer_stride, int precision,
                             int* pStop) {
    if (!inAmp || !inD || !qs || !intensities || !dirs) return fail(DPX_ERR_ARG, "NULL buffer");
    int grid_size;
    double qmax;
    if (int rc = grid_from_voxels(voxels, thDivs, phDivs, stepSz, &grid_size, &qmax)) return rc;
    if (pStop && *pStop) return fail(DPX_ERR_STOPPED, "stopped");
    int dev = 0;
    cudaGetDevice(&dev);
    dpx_ctx ctx;
    if (int rc = dpx_ctx_create(dev, &ctx)) return rc;
    dpx_grid g;
    int rc = dpx_grid_create(ctx, grid_size, qmax, precision, &g);
    if (rc) { dpx_ctx_destroy(ctx); return rc; }
    rc = dpx_grid_write(g, inAmp, inD);
    if (!rc)
        rc = dpx_orientation_average(ctx, 1, &g, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, qPoints, qs, dirs,
                                     0, dir_layer_stride, maxIters, convergence, intensities);
    if (!rc && pStop && *pStop) rc = fail(DPX_ERR_STOPPED, "stopped");
    dpx_grid_destroy(g);
    dpx_ctx_destroy(ctx);
    return rc;
}

}  // extern "C"

namespace {

// Shared body of the host-buffer assembly drop-ins: source grids from host
// (values, derivatives) pairs, destination from outData (values only), one
// dpx_grid_assemble, values copied back.  accumulate = 0 starts from zero
// (GPUSumGridsJacobSphr overwrites its output).
int assemble_host(int64_t voxels, int thDivs, int phDivs, double stepSize, int n, const double* const* inAmp,
                  const double* const* inD, const double* rot, const double* tr, const int* n_copies,
                  const double* copy_rot, const double* copy_tr, const double* sym_scale, const double* lattice,
                  double scale, double* outData, bool accumulate, int precision, int* pStop) {
    if (!outData || !inAmp || !inD || n <= 0) return fail(DPX_ERR_ARG, "NULL buffer");
    for (int m = 0; m < n; ++m)
        if (!inAmp[m] || !inD[m]) return fail(DPX_ERR_ARG, "NULL source grid");
    int grid_size;
    double qmax;
    if (int rc = grid_from_voxels(voxels, thDivs, phDivs, stepSize, &grid_size, &qmax)) return rc;
    if (pStop && *pStop) return fail(DPX_ERR_STOPPED, "stopped");
    int dev = 0;
    cudaGetDevice(&dev);
    dpx_ctx ctx;
    if (int rc = dpx_ctx_create(dev, &ctx)) return rc;
    std::vector<dpx_grid> src(n, nullptr);
    dpx_grid dst = nullptr;
    int rc = dpx_grid_create(ctx, grid_size, qmax, precision, &dst);
    for (int m = 0; m < n && !rc; ++m) {
        rc = dpx_grid_create(ctx, grid_size, qmax, precision, &src[m]);
        if (!rc) rc = dpx_grid_write(src[m], inAmp[m], inD[m]);
    }
    if (!rc && accumulate) rc = dpx_grid_write(dst, outData, nullptr);
    if (!rc) rc = dpx_grid_assemble(dst, n, src.data(), rot, tr, n_copies, copy_rot, copy_tr, sym_scale, lattice, scale);
    if (!rc) rc = dpx_grid_read(dst, outData, nullptr);
    if (!rc && pStop && *pStop) rc = fail(DPX_ERR_STOPPED, "stopped");
    for (dpx_grid g : src)
        if (g) dpx_grid_destroy(g);
    if (dst) dpx_grid_destroy(dst);
    dpx_ctx_destroy(ctx);
    return rc;
}

}  // namespace

extern "C" {

int dpx_calc_man_sym_jacob_sphr(int64_t voxels, int thDivs, int phDivs, int numCopies, double stepSize,
                                const double* inModel, double* outData, const double* ds, const double* locX,
                                const double* locY, const double* locZ, const double* locA, const double* locB,
                                const double* locC, double scale, int precision, int* pStop) {
    if (numCopies <= 0) return fail(DPX_ERR_ARG, "numCopies must be positive");
    if (!locX || !locY || !locZ || !locA || !locB || !locC) return fail(DPX_ERR_ARG, "NULL location array");
    // entry 0 places the inner object; entries 1..numCopies are the copies
    const double rot[3] = {locA[0], locB[0], locC[0]}, tr[3] = {locX[0], locY[0], locZ[0]};
    std::vector<double> crot(3 * (size_t)numCopies), ctr(3 * (size_t)numCopies);
    for (int k = 0; k < numCopies; ++k) {
        crot[3 * k] = locA[k + 1];
        crot[3 * k + 1] = locB[k + 1];
        crot[3 * k + 2] = locC[k + 1];
        ctr[3 * k] = locX[k + 1];
        ctr[3 * k + 1] = locY[k + 1];
        ctr[3 * k + 2] = locZ[k + 1];
    }
    return assemble_host(voxels, thDivs, phDivs, stepSize, 1, &inModel, &ds, rot, tr, &numCopies, crot.data(),
                         ctr.data(), &scale, nullptr, 1.0, outData, true, precision, pStop);
}

int dpx_calc_spc_fill_sym_jacob_sphr(int64_t voxels, int thDivs, int phDivs, double stepSize, const double* inModel,
                                     double* outData, const double* ds, const double* vectorMatrix,
                                     const double* repeats, const double* innerRots, const double* innerTrans,
                                     double scale, int precision, int* pStop) {
    if (!vectorMatrix || !repeats || !innerRots || !innerTrans) return fail(DPX_ERR_ARG, "NULL lattice argument");
    // SymmetryGenJacob.cu:83-125 multiplies by sum_n e^{-i n q.a}, the complex
    // conjugate of GridSymmetry::calcAmplitude's sum_n e^{+i n q.a}; the same
    // lattice sum over -a reproduces it
    double lat[12];
    for (int k = 0; k < 9; ++k) lat[k] = -vectorMatrix[k];
    for (int k = 0; k < 3; ++k) lat[9 + k] = repeats[k];
    return assemble_host(voxels, thDivs, phDivs, stepSize, 1, &inModel, &ds, innerRots, innerTrans, nullptr, nullptr,
                         nullptr, nullptr, lat, scale, outData, true, precision, pStop);
}

int dpx_sum_grids_jacob_sphr(int64_t voxels, int thDivs, int phDivs, double stepSz, const double* const* inAmpData,
                             const double* const* inD, const double* trans, const double* rots, int numGrids,
                             double* outAmpData, int precision, int* pStop) {
    if (numGrids <= 0 || !trans || !rots) return fail(DPX_ERR_ARG, "bad grid list");
    return assemble_host(voxels, thDivs, phDivs, stepSz, numGrids, inAmpData, inD, rots, trans, nullptr, nullptr,
                         nullptr, nullptr, nullptr, 1.0, outAmpData, false, precision, pStop);
}

}  // extern "C"
