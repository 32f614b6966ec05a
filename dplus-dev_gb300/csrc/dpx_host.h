// dpx_host.h — host-side internals shared by the libdpx translation units
// (dpx_api.cpp, dpx_batch.cpp, dpx_server.cpp): the context and grid handles,
// status helpers and the staging routines.  Not part of the C-ABI.
#pragma once
#include "dpx.h"
#include "dpx_internal.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

namespace dpxh {

// Records the per-thread message returned by dpx_last_error; returns code.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* where);

#define DPX_CUDA(call)                                              \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return dpxh::cuda_fail(e_, #call);   \
    } while (0)

constexpr double kPi = 3.14159265358979323846;

// Grow-only device buffer owned by a context.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

// Grow-only pinned host staging buffer owned by a context.  get() waits for
// the copy that last read it (the event recorded by copied()) before handing
// it out again.
struct HostPinned {
    void* p = nullptr;
    size_t bytes = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
    cudaError_t get(size_t n, char** out) {
        if (pending) {
            if (cudaError_t e = cudaEventSynchronize(done)) return e;
            pending = false;
        }
        if (n > bytes) {
            if (p) cudaFreeHost(p);
            p = nullptr;
            bytes = 0;
            if (cudaError_t e = cudaMallocHost(&p, n)) return e;
            bytes = n;
        }
        *out = static_cast<char*>(p);
        return cudaSuccess;
    }
    // the stream's copies out of the buffer have been issued
    cudaError_t copied(cudaStream_t s) {
        if (!done)
            if (cudaError_t e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming)) return e;
        if (cudaError_t e = cudaEventRecord(done, s)) return e;
        pending = true;
        return cudaSuccess;
    }
    void release() {
        if (pending && done) cudaEventSynchronize(done);
        if (p) cudaFreeHost(p);
        if (done) cudaEventDestroy(done);
        p = nullptr;
        done = nullptr;
        bytes = 0;
        pending = false;
    }
};

}  // namespace dpxh

struct dpx_ctx_s {
    int device = 0;
    int refs = 1;  // the caller's handle + one per live grid / batch / server
    bool closed = false;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    int fill_cpt = 8, fill_threads = 128;  // FP32 fill shape (dpx_autotune_fill)
    bool fill_persistent = false;
    int fill_poly = 0;  // phi columns per work item whose sincos run on the FMA pipe
    int fill_method = 1;  // DPX_FILL_HARMONIC (default) / DPX_FILL_DIRECT
    int conv_rule = 0;              // DPX_CONV_CPU (default) / DPX_CONV_GPU (dpx_ctx_set_convergence)
    int64_t conv_samples = 8192;    // samples per step of DPX_CONV_GPU
    // stage timing of the last harmonic fill (dpx_ctx_set_timing): events
    // around the moments of the atoms and of the voxels, the synthesis and the
    // whole fill; the points and K of that fill
    bool timing = false;
    cudaEvent_t tev[8] = {};
    int tev_used = 0;
    double stage_points = 0, stage_k = 0;
    // with timing on, events around the last orientation average's main kernel
    cudaEvent_t aev[2] = {};
    bool aev_used = false;
    dpxh::DevBuf atoms, table, ions, models, groups, plan, partial, result, dirs, debye;
    dpxh::DevBuf harmonic; // the harmonic fill's launch scratch
    dpxh::DevBuf dirsort;  // the average's angular-order scratch
    dpxh::DevBuf direct;   // the FP64 direct sum's tables and partial amplitudes
    std::vector<char> host_stage;
};

struct dpx_grid_s {
    dpx_ctx ctx;
    int grid_size;
    double qmax;
    int precision;
    dpx::Geom g;
    void* cells;
    // the phi-spline derivatives match the values: set by a fill that writes
    // them (the harmonic synthesis) and by dpx_grid_compute_splines, cleared
    // by every other write and whenever the device pointer is handed out
    bool splines_current = false;
};

namespace dpxh {

int set_device(dpx_ctx ctx);
void ctx_retain(dpx_ctx ctx);
void ctx_release(dpx_ctx ctx);
size_t cell_bytes(int precision);
extern const int kFillShape[][4];
extern const int kFillShapes;

// Unique-ion form factors minus the dummy-atom solvent for shells 0..Lp, [U][Lp+1].
void aff_table(int U, const int* api, const double* coeffs, const double* rads, int flags, double sol_ed,
               double c1, int Lp, double step, std::vector<double>& out);
// The same at the nq values q[k], [U][nq].
void aff_at(int U, const int* api, const double* coeffs, const double* rads, int flags, double sol_ed, double c1,
            int nq, const double* q, std::vector<double>& out);
// A leaf's form factors on shells 0..Lp, [U][Lp+1]: its tabulated ones
// (dpx_pdb_desc::aff) or aff_table of its coefficients.  check_leaf_grid
// rejects a tabulated leaf whose table is shorter than the grid's shells.
void leaf_aff_table(const dpx_pdb_desc& d, int Lp, double step, std::vector<double>& out);
int check_leaf_grid(const dpx_pdb_desc& d, const dpx::Geom& G);
// Tait-Bryan X1Y2Z3 rotation (EulerD).
void euler(double a, double b, double c, double R[9]);
int check_pdb(const dpx_pdb_desc& d);
// grid_size and qmax of the reference's (voxels, thDivs, phDivs, stepSize)
// description of a Jacobian sphere grid (voxels = complex cells).
int grid_from_voxels(int64_t voxels, int thDivs, int phDivs, double stepSize, int* grid_size, double* qmax);

// Model structs of one average and their docked-copy group tables.  build_models
// stages the tables on the host (gstage) with offsets; place_models points the
// structs at the tables' device copy.
struct ModelTables {
    std::vector<dpx::ModelDev> md;
    std::vector<char> gstage;
    std::vector<size_t> oR, oT, oO, oS, oA, oW, oF;
};
int build_models(int n_models, const void* const* cells, const double* rot, const double* tr, const int* n_copies,
                 const double* copy_rot, const double* copy_tr, const double* sym_scale, ModelTables& t);
void place_models(ModelTables& t, char* dbase);
// Model structs for the kernels; group tables staged in gstage for ctx->groups.
int prepare_models(dpx_ctx ctx, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                   const int* n_copies, const double* copy_rot, const double* copy_tr, const double* sym_scale,
                   std::vector<dpx::ModelDev>& md, std::vector<char>& gstage);

// Device tables of one leaf in a staging buffer (offsets from its start).
struct LeafTables {
    size_t atoms = SIZE_MAX;  // SIZE_MAX: the caller's device atoms
    size_t off = 0, aff = 0, pref = 0, boxes = SIZE_MAX;
    int64_t items = 0, n_boxes = 0;
    double cen[3] = {0, 0, 0};
    double origin = 0;  // F(0) = scale (sum_u aff_u(0) N_u + sum_b w_b V_b), FP64
};
// Appends leaf d's tables for grid G (FP32 with cpt cells per item, or FP64).
// direct_boxes = false leaves the boxes out of the staging and out of F(0):
// the harmonic fill reads them from the descriptor and adds
// scale * box_volume_sum(d) to F(0) while its moments run.
void stage_leaf(std::vector<char>& h, const dpx_pdb_desc& d, const dpx::Geom& G, bool fp32, int cpt, LeafTables& t,
                bool direct_boxes = true);
// sum_b w_b Lx_b Ly_b Lz_b over d's solvent boxes, in their order, FP64.
double box_volume_sum(const dpx_pdb_desc& d);
// The FP32 fill job of a staged leaf whose buffer sits at device address dbase.
dpx::FillJob make_job(const dpx_pdb_desc& d, const LeafTables& t, const char* dbase, const dpx::Geom& G, void* grid,
                      int64_t tile_start);
// Harmonic (multipole) FP32 fill of one leaf (dpx_harmonic_host.cpp), planned
// once and launched any number of times.  harmonic_plan (host work and
// synchronizations on stream st) returns DPX_OK, a negative status, or
// kHarmDeclined when the method does not take the leaf (boxes without their
// voxel step, orders or radial bins beyond the kernels' limits): the caller
// then fills with the direct sum.  The plan owns a device arena (stream-ordered
// on st) with its tables and point sets; harmonic_launch queues only kernels
// and memsets, so a graph can record it.
constexpr int kHarmDeclined = 1;
struct HarmPlan {
    dpx::Geom G{};
    cudaStream_t stream = nullptr;  // the arena is freed on it
    int nbins = 0, LM = 0, K = 0;
    double delta = 0.0;
    int64_t n_vox = 0;
    int n_units[2] = {0, 0}, n_groups[2] = {0, 0};  // [0] atoms, [1] solvent voxels
    int n_parts[2] = {0, 0};  // CTAs of the tensor-core moments per set
    double cen[3] = {0, 0, 0};   // the centring translation restored per cell
    float scale = 1.f, vox_s = 0.f;
    double origin = 0.0;         // F(0), FP64, scaled
    double stage_points = 0.0, stage_k = 0.0;  // points and mean (l, m) per point (stage timing)
    char* arena = nullptr;
    size_t arena_bytes = 0;
    size_t o_lmax = 0, o_lmb = 0, o_ab = 0, o_cr = 0, o_nmm = 0, o_nodes = 0, o_vinv = 0, o_aff = 0;
    size_t o_pts[2] = {0, 0}, o_units[2] = {0, 0}, o_groups[2] = {0, 0}, o_gu[2] = {0, 0};
    // scratch of a launch (offsets from the caller's scratch, 256-byte aligned)
    size_t s_MP[2] = {0, 0}, s_M[2] = {0, 0}, s_C[2] = {0, 0};
    size_t scratch_bytes = 0;
    size_t o_job = 0;       // the plan's own job (scratch and grid at offset 0) in the arena
    size_t o_T = 0;         // the radial tables T_n(i, b, l) in the arena (computed when planned)
    dpx::HarmShape shape{};  // its launch layout
};
// The stream of a launch; tev (null: no timing) receives the stage events.
struct HarmStreams {
    cudaStream_t st = nullptr;
    cudaEvent_t* tev = nullptr;
};
int harmonic_plan(cudaStream_t st, const dpx_pdb_desc& d, const dpx::Geom& G, HarmPlan& p);
void harmonic_plan_release(HarmPlan& p);
// Fills grid (FP32 cells with their phi-spline derivatives) from the plan.
int harmonic_launch(const HarmStreams& S, const HarmPlan& p, void* scratch, float4* grid);
// Kernel launches of one harmonic_launch.
int harmonic_launches(const HarmPlan& p);
// The device job of a plan with its scratch at scratch_off from a launch's
// scratch base and its grid at grid_off from the launch's grid base (the
// block layout is set by dpx::plan_harmonic_jobs over the job table).
dpx::HarmJob harmonic_job(const HarmPlan& p, size_t scratch_off, size_t grid_off);
// The context's stream for a harmonic launch and the stage-timing events when
// timing is on (created on first use, so call it outside stream capture);
// ctx_stage_record keeps the plan's figures for dpx_ctx_stage_times.
int ctx_harmonic_streams(dpx_ctx ctx, HarmStreams& S);
void ctx_stage_record(dpx_ctx ctx, const HarmPlan& p);
// The FP64 fill launch of a staged leaf.
cudaError_t launch_leaf_f64(cudaStream_t s, const dpx_pdb_desc& d, const LeafTables& t, const char* dbase,
                            const dpx::Geom& G, void* grid);

// Bracket tables of one orientation average (IntegrateLayersTogether).
struct Brackets {
    std::vector<int> layer, off{0}, qidx;
    std::vector<double> q;
    int max_q = 1;
};
void make_brackets(const dpx::Geom& G, int grid_size, double qmax, int nq, const double* Q, Brackets& b);

}  // namespace dpxh
