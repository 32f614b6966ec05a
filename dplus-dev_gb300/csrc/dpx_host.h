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
    // the harmonic fill's radial tables and atoms' set run on aux beside the
    // voxels' moments: aux waits for aux_go (the plan's upload), the voxels'
    // contractions for aux_done (the tables), the synthesis for aux_atoms
    cudaStream_t aux = nullptr;
    cudaEvent_t aux_go = nullptr, aux_done = nullptr, aux_atoms = nullptr;
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
    dpxh::DevBuf atoms, table, ions, models, groups, plan, partial, result, dirs, debye, harmonic;
    dpxh::DevBuf voxels;   // the harmonic fill's voxels, binned
    dpxh::DevBuf dirsort;  // the average's angular-order scratch
    dpxh::DevBuf direct;   // the FP64 direct sum's tables and partial amplitudes
    dpxh::HostPinned pin_plan, pin_totals, pin_small, pin_units, pin_atomset;  // the harmonic fill's host staging
    std::vector<dpxh::DevBuf> leaf_boxes;  // the harmonic fill's solvent boxes, per leaf of a batch
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
// Tait-Bryan X1Y2Z3 rotation (EulerD).
void euler(double a, double b, double c, double R[9]);
int check_pdb(const dpx_pdb_desc& d);

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
// Harmonic (multipole) FP32 fill of a staged leaf (dpx_harmonic_host.cpp).
// harmonic_accepts decides before the staging: boxes need their voxel step,
// and the expansion order and the radial bins must stay within the kernels'
// limits (device atoms are copied to `host_atoms` to measure them).  It
// stages the leaf's solvent boxes on the device (context buffer `slot`:
// centred, counted) and fills `hl`: the radius of the point sets about the
// leaf's centre, the voxel total and the staged arrays harmonic_fill bins.
struct HarmLeaf {
    double R = 0.0;      // bounds the atoms and the solvent boxes' corners
    double R_pts = 0.0;  // bounds the atoms and the voxel centres (<= R)
    int64_t nb = 0, nv = 0;
    const float4* boxes = nullptr;
    const int64_t* counts = nullptr;
    int64_t* vstart = nullptr;
    int64_t* run_sums = nullptr;
};
bool harmonic_accepts(dpx_ctx ctx, int slot, const dpx_pdb_desc& d, const dpx::Geom& G,
                      std::vector<float>& host_atoms, HarmLeaf& hl, int* status);
int harmonic_fill(dpx_ctx ctx, const dpx_pdb_desc& d, const LeafTables& t, const char* dbase, const dpx::Geom& G,
                  void* grid, const std::vector<float>& host_atoms, const HarmLeaf& hl);
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
