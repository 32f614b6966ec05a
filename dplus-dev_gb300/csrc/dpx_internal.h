// dpx_internal.h — shared declarations between the host side (dpx_api.cpp)
// and the sm_103a kernels (dpx_kernels.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dpx {

// Jacobian sphere grid geometry (D+ Grid.cpp:169-200): shell i in 1..Lp holds
// (3i+1) theta rows of 6i phi points; cell 0 is the origin.
struct Geom {
    int L;        // radial layers (grid_size / 2)
    int Lp;       // layers including the 3 extra shells
    double step;  // qmax / L
    int64_t P;    // complex cells
};

inline Geom make_geom(int grid_size, double qmax) {
    Geom g;
    g.L = grid_size / 2;
    g.Lp = g.L + 3;
    g.step = qmax / double(g.L);
    int64_t lp = g.Lp;
    g.P = 6 * lp * (lp + 1) * (lp + 1) + 1;
    return g;
}

__host__ __device__ inline int64_t shell_base(int64_t i) { return 1 + 6 * (i - 1) * i * i; }

// Cells per work item of the FP64 fill (the FP32 fill takes it from the context).
constexpr int kFill64Cells = 2;

// One placed view of a grid for the orientation average: the leaf's own
// rotation/translation and, for a docked assembly, groups of copies that share
// a rotation (ManualSymmetry translationsPerOrientation).
struct ModelDev {
    const void* grid;      // float4* (FP32) or double4_32a* (FP64): {re, im, dre, dim} per cell
    double R[9];           // leaf RotMat (row-major)
    double tr[3];          // leaf translation
    int n_groups;          // 0 = plain leaf
    const double* group_R; // [9 n_groups] rotation per group (row-major)
    const int* group_off;  // [n_groups + 1] into trans
    const double* trans;   // [3 K]
    const double* group_step;  // [3 n_groups] d of a group whose translations are t0 + m d
    const int* group_ap;       // [n_groups] M of such a group (0: an arbitrary list)
    // FP32 average geometry: per group C = R_copy R_leaf as floats (row-major)
    // and w = C t_leaf; for a model without groups Rf = R_leaf and w = R_leaf t_leaf
    const float* group_Cf;     // [9 n_groups]
    const double* group_w;     // [3 n_groups]
    float Rf[9];
    double w[3];
    double sym_scale;
    int plain;             // R is the identity and tr is zero
};

struct AvgPlan {
    int n_brackets;
    const int* br_layer;     // [nbr] layer index of the bracket
    const int* br_q_off;     // [nbr + 1] offsets into br_q / br_qidx
    const double* br_q;      // q values, bracket-major
    const int* br_qidx;      // index into the result vector
    int max_q;               // max q per bracket
    const double* dirs;      // [D x 2] theta, phi
    int64_t dir_stride;      // per-layer stride in directions (0 = shared)
    int64_t n_samples;       // samples per bracket
    int chunk;               // samples per chunk
    int chunk_off;           // first chunk holds chunk - chunk_off samples
    int64_t n_chunks;
    double* partial;         // [nbr][n_chunks][max_q] partial sums, then 5 nbr max_q doubles of
                             // scratch: the average's bracket tables, then the finalize's sums
    int need_dir;            // some model is placed or docked: the kernel needs the direction vector
    int one_leaf;            // one model without docked copies (ModelDev::n_groups == 0): with a
                             // shared direction set the average slides its plane window
    int* sort_scratch;       // dir_sort_bytes(n_samples) of device scratch, or nullptr: with eps = 0
                             // and a shared direction set the samples are taken in an angular order
                             // (the mean is the same; neighbouring threads gather neighbouring cells)
    const int* dir_order;    // the sample order in use (set by launch_average; nullptr: as given)
    int conv_group;          // eps > 0 only.  0: the reference CPU's convergence test (4-column history
                             // every 100 samples, AverageIntensitiesBetweenLayers); > 0: the reference
                             // GPU paths' test (OAJacob.cu:320-337, GPUHybridCalc.cu:705-720) on steps of
                             // conv_group chunks: after 4 steps, every q of the bracket within eps of its
                             // mean at each of the 3 steps before
};
// Bytes of AvgPlan::sort_scratch for n samples.
size_t dir_sort_bytes(int64_t n);

// host helpers (dpx_api.cpp)
void q_brackets(int grid_size, double qmax, int nq, const double* Q, int* layer_of_q);
int set_error(int code, const char* msg);  // records the per-thread message, returns code

// amplitude fill (dpx_fill.cu).  fill_items writes the work-item prefix
// pref[0..Lp] (origin, then per shell (floor(3i/2)+1) rows x ceil(3i/cpt)
// column chunks) and returns the item count.
int64_t fill_items(const Geom& g, int cpt, int64_t* pref);

// One structure on one grid in a batched FP32 fill.  Its items occupy tiles
// [tile_start, tile_start + ceil(n_items / threads)); jobs are in ascending
// tile_start order.
struct FillJob {
    const float4* atoms;    // centred, sorted by ion
    const int* ion_off;     // [U + 1]
    const float* aff_f32;   // [U][Lp + 1]
    const int64_t* pref;    // [Lp + 1] item prefix
    const float4* boxes;    // [2 n_boxes]: {cx, cy, cz, weight}, {Lx, Ly, Lz, 0} (centred, nm, e/nm^3)
    float4* grid;
    int64_t n_items;
    int64_t tile_start;
    double step;
    double cx, cy, cz;
    double origin;          // F(q = 0), summed in FP64 on the host (every term adds in phase there)
    int U, Lp, use_center;
    int n_boxes;
    float scale;
};
// One launch over every tile of every job: persistent (one CTA per resident
// slot, atomic tile counter d_counter) or flat (one CTA per tile).  boxes: some
// job carries voxelized-solvent boxes (always the flat form, box code compiled in).
cudaError_t launch_fill_f32_batch(cudaStream_t s, const FillJob* d_jobs, int n_jobs, int64_t total_tiles,
                                  unsigned long long* d_counter, int cells_per_thread, int block, int poly,
                                  bool persistent, bool boxes);
cudaError_t launch_fill_f64(cudaStream_t s, const float4* atoms, const int* ion_off, int U, const double* aff,
                            const Geom& g, const int64_t* d_pref, int64_t n_items, const double center[3],
                            double scale, const float4* boxes, int n_boxes, double4_32a* grid);

// VEGAS (dpx_kernels.cu): points of one iteration of one bracket, then the
// single-block reduction / bin refinement / running mean / convergence test.
cudaError_t launch_vegas_points(cudaStream_t s, bool fp64, const Geom& g, int n_models, const ModelDev* d_models,
                                int need_dir, const double* d_q, int m, int ppi, uint64_t seed, uint64_t key,
                                const double* d_bounds, const int* d_done, double* d_I);
cudaError_t launch_vegas_update(cudaStream_t s, double* d_bounds, const double* d_I, int m, int ppi, int it,
                                double eps, double* d_hist, int* d_done, double* d_res, const int* d_qidx);

// Gauss-Kronrod: one phi interval of one theta node of one q.
struct GKTask {
    double q, st, ct, pmin, pmax;
};
cudaError_t launch_gk_phi(cudaStream_t s, bool fp64, const Geom& g, int n_models, const ModelDev* d_models,
                          const GKTask* d_tasks, int n, double2* d_kg);

// Grid-path assembly: dst += scale * lattice * sum of models (GetCart path).
// lattice: NULL or {a[3], b[3], c[3], Na, Nb, Nc}.
cudaError_t launch_assemble(cudaStream_t s, bool fp64, const Geom& g, int n_models, const ModelDev* d_models,
                            const double* lattice, double scale, void* dst);

// other kernels (dpx_kernels.cu)
cudaError_t launch_splines_f32(cudaStream_t s, const Geom& g, float4* grid);
cudaError_t launch_splines_f64(cudaStream_t s, const Geom& g, double4_32a* grid);
// Directions per thread of the FP32 slide average (1 or 2; -1: other values).
int set_average_dpt(int dpt);
// One solve of a batched average (launch_average_batch): a plain leaf on its
// grid with its own brackets and partial-sum region, every solve on the same
// shared direction set (plan.dir_order: its angular order, or nullptr).
struct AvgJob {
    AvgPlan plan;
    const ModelDev* model;  // the plain leaf (identity placement) on its grid
    double* res;            // [nq] I(q)
    double step;            // the grid's radial step
    int Lp;
    int origin;             // the first q is 0: res[0] = |F(0)|^2 from the origin cell
    int seg_len, n_seg;     // set by plan_average_batch
    int64_t bx;             // blocks along the chunks (plan_average_batch)
    int64_t block0;         // the solve's first block in the batched average (plan_average_batch)
};
// Host: the launch shape of every job; returns the total blocks of the average.
int64_t plan_average_batch(AvgJob* jobs, int n, bool fp64);
// Bracket tables, average and finalize (with the q = 0 terms) of n_jobs solves
// in three launches; max_brackets = the largest n_brackets.
cudaError_t launch_average_batch(cudaStream_t s, bool fp64, const AvgJob* d_jobs, int n_jobs, int max_brackets,
                                 int64_t total_blocks, double eps);
// The angular order of a shared direction set (dir_sort_bytes(n) of scratch),
// or nullptr when the set is too small to sort.
const int* launch_dir_order(cudaStream_t s, const double* dirs, int64_t n, int* scratch);
// kev (optional): two events recorded just before and after the main average kernel
cudaError_t launch_average(cudaStream_t s, bool fp64, const Geom& g, int n_models, const ModelDev* d_models,
                           const AvgPlan& plan, cudaEvent_t* kev = nullptr);
cudaError_t launch_finalize(cudaStream_t s, const AvgPlan& plan, double eps, double* d_res);
// SFU calibration: blocks x 256 threads x iters x 8 __sincosf (2 MUFU ops each)
cudaError_t launch_sfu_probe(cudaStream_t s, int blocks, int iters, float* out);

// Harmonic (multipole) FP32 fill of one leaf (dpx_harmonic.cu).  Points are
// float4 (x, y, z nm about the centre, weight), sorted by group (radial bin,
// and ion for atoms); a unit is <= 1024 points of one group.
// One structure's harmonic fill in the batched launches (launch_harmonic_jobs).
// Table pointers are absolute (the structure's plan arena); scratch and grid
// are byte offsets from the launch's scratch and grid bases, so one table
// serves any scratch and grid.  Set 0: atoms, set 1: solvent voxels.
// Tensor-core moments (hm_moments_tc): the (l, m) steps of a unit whose bin
// carries orders l <= LM, laid out as octets o of the orders m = 8o .. 8o + 7
// (octet o takes LM + 1 - 8o steps: step d holds l = m + d for each of its
// orders m), cut evenly over 4 P producer-warp slots of at most
// kTcSlotSteps steps each, P CTAs per unit.  units[].w holds a unit's first
// CTA within its set.
constexpr int kTcSlotSteps = 48;
__host__ __device__ inline int tc_octet_first(int LM, int o) { return o * (LM + 1) - 4 * o * (o - 1); }
__host__ __device__ inline int tc_steps(int LM) { return tc_octet_first(LM, LM / 8 + 1); }
__host__ __device__ inline int tc_parts(int LM) { return (tc_steps(LM) + 4 * kTcSlotSteps - 1) / (4 * kTcSlotSteps); }
// Which moments kernel the harmonic launches use (process-wide): 0 tcgen05.mma
// (FP16 hi + lo operands, accumulators in tensor memory), 1 mma.sync TF32
// m16n8k8, 2 (the default) mma.sync FP16 m16n8k16 (split operands, sums in
// shared memory).
void set_moments_kernel(int kind);
int moments_kernel();
// Faults recorded by the tensor-core moments kernel (a wait that ran past its
// limit): reads and clears the device flag (synchronous).
cudaError_t harmonic_take_faults(unsigned* flags);

struct HarmJob {
    int Lp, nbins, LM, K;
    double step, delta;        // q step, radial bin width (nm)
    const int* lmax;           // [Lp+1] l_i
    const int* lmb;            // [nbins] the orders a bin needs (<= LM)
    const double* nodes;       // [6] Chebyshev nodes on [-1, 1]
    const double* vinv;        // [6][6] inverse Vandermonde of the nodes
    const float2* ab;          // [K] Legendre recurrence coefficients
    const float2* cr;          // [K] scaled recurrence {c_lm, r_lm} (moments)
    const float* nmm;          // [LM+1] Pbar_mm = nmm[m] (-sin theta)^m
    const float* aff;          // [U][Lp+1] ion form factors (atoms)
    const float4* pts[2];
    const int4* units[2];      // {first point, count, bin, 0}
    const int2* groups[2];     // {bin, ion or -1}
    const int* gu[2];          // [G+1] first unit of each group
    int n_units[2], G[2];
    int n_parts[2];            // CTAs of the tensor-core moments per set (sum over units of tc_parts)
    int vox;                   // the voxel set exists
    int use_center;
    float vox_s, scale;        // voxel edge (nm), scale
    double cx, cy, cz;         // the centring translation restored per cell
    double origin;             // F(0)
    const float* T;            // radial polynomial tables T_n(i, b, l), computed when planned
    size_t s_MP[2], s_M[2], s_C[2];  // scratch offsets (bytes)
    size_t grid_off;           // grid offset (bytes)
    float4* grid_ptr;          // the grid itself when not null (grid_off unused)
    // the job's first blocks in each launch (plan_harmonic_jobs)
    int64_t b_mom[2], b_grp[2], b_con[2], b_syn;
};
// Blocks of the launches and the largest shell count and order (shared
// memory) of a job table.
struct HarmShape {
    int64_t moments, groups, contract, synth;
    int maxLp, maxLM;
    int moments_kind;  // moments_kernel() when planned
    cudaError_t reserve_error;  // raising the launches' shared-memory limits (on the planning device)
};
// Host: the block layout of n jobs (sets their b_* fields).
HarmShape plan_harmonic_jobs(HarmJob* jobs, int n);
// The harmonic fills of n jobs in four launches: moments, group sums,
// contraction, synthesis (the radial tables are the plans').  ev[0..1] (when
// not null) are recorded around the moments, ev[2..3] around the synthesis.
cudaError_t launch_harmonic_jobs(cudaStream_t s, const HarmJob* d_jobs, int n, const HarmShape& sh, char* scratch,
                                 char* grid, cudaEvent_t* ev);
int harmonic_launches_per_batch();
// The radial tables of a plan (once per plan): j_l at the Chebyshev nodes of
// every (shell i >= 1, bin) in FP64 into Jn [(Lp + 1) nbins 6 (LM + 1)], then
// the interpolation coefficients T [(Lp + 1) nbins (LM + 1) 8] (FP32).
struct RadialTableArgs {
    int Lp, nbins, LM;
    double step, delta;
    const int* lmax;
    const double* nodes;
    const double* vinv;
    double* Jn;
    float* T;
};
cudaError_t launch_radial_tables(cudaStream_t s, const RadialTableArgs& a);
int harmonic_max_l();
int harmonic_nodes();
int harmonic_max_bins();
// Solvent boxes expanded into voxels and sorted by radius bin on the device.
// Boxes per run of the voxel-start scan (launch_voxel_bins); VoxelBinArgs::run_sums
// holds ceil(nb / kVoxelScanRun) entries.
constexpr int kVoxelScanRun = 1024;
// A leaf's raw solvent boxes staged on the device: centred, counted, and R.
struct VoxelPrepArgs {
    const float* raw;       // [8 nb] D+ box records
    int64_t nb;
    double cx, cy, cz;      // the leaf's centre
    float vs;               // voxel edge (nm)
    float4* boxes;          // out [2 nb] {centre - c, w}, {L, 0}
    int64_t* counts;        // out [nb] voxels per box
    unsigned long long* scal;  // out {bits of the largest squared corner distance (FP32), total voxels,
                               //      bits of the largest squared voxel-centre distance (FP32)}
};
cudaError_t launch_voxel_prepare(cudaStream_t s, const VoxelPrepArgs& a);
struct VoxelBinArgs {
    const float4* boxes;    // [2 nb] {cx, cy, cz, w} about the centre, {Lx, Ly, Lz, 0}
    const int64_t* counts;  // [nb] voxels per box
    int64_t* vstart;        // [nb] first voxel of each box (written)
    int64_t* run_sums;      // [ceil(nb / kVoxelScanRun)] scratch of the vstart scan
    int64_t nb, nv;
    float vs, delta;        // voxel edge, bin width (nm)
    int nbins;
    float4* tmp;            // [nv] voxels in box order
    int* vbin;              // [nv] their bins
    int* hist;              // [nbins][blocks]
    int64_t* off;           // [nbins][blocks]
    int64_t* total;         // [nbins]
    float4* out;            // [nv] voxels sorted by bin
};
cudaError_t launch_voxel_bins(cudaStream_t s, const VoxelBinArgs& a);
// Raises hm_moments' and hm_synth's dynamic shared-memory limits on the current
// device to what a fill of shells up to Lp and orders up to LM needs (never
// lowers them).  Called when a fill is planned, outside any stream capture;
// the launches below do not touch the limits.
cudaError_t harmonic_reserve_smem(int Lp, int LM);
// Pipe calibration kernels: kind 0 scalar FP32 FMA, 1 packed f32x2 FMA, 2
// mma.sync m16n8k8 TF32 (256 threads a block, iters steps of 8 / 8 / 4
// independent operations per thread or warp).
cudaError_t launch_pipe_probe(cudaStream_t s, int kind, int blocks, int iters, float* out);
// cycles[2]: one thread issuing tc_issue_probe_mmas() tcgen05 MMAs (M = 128,
// N = 16 and N = 256) until their commit completes; *status 1 on a wait limit.
cudaError_t launch_tc_issue_probe(cudaStream_t s, long long* cycles, int* status);
int tc_issue_probe_mmas();

// Debye sum of one leaf (dpx_debye.cu).  Atoms padded to a multiple of the
// 128-atom tile; F tables [nq][npad] of the path's type; partial sums
// [debye_pair_blocks(npad)][nq].
struct DebyeArgs {
    const float4* pos;      // [npad] (x, y, z, 0) nm, padding zero
    const int* ion;         // [n] ion index per atom
    const float* bfactor;   // [n] B factors (Debye-Waller) or nullptr
    const float2* anom;     // [n] (f', f'') or nullptr
    const double* ff;       // [U][nq] ion form factors minus the dummy-atom solvent
    const double* q;        // [nq]
    void* Fr;               // [nq][npad] per-atom form factors (real part)
    void* Fi;               // [nq][npad] imaginary part (anomalous only)
    double* partial;        // [pair blocks][nq]
    double* out;            // [nq]
    int64_t n, npad;
    int nq;
    double scale2;          // I is multiplied by scale^2
};
int64_t debye_padded_atoms(int64_t n);
int debye_pair_blocks(int64_t npad);
cudaError_t launch_debye(cudaStream_t s, bool fp64, bool anomalous, const DebyeArgs& a);
// d_res[0] = |origin cell|^2 (I at q = 0 of one plain leaf)
cudaError_t launch_origin_intensity(cudaStream_t s, bool fp64, const void* grid, double* d_res);
// d_res[0] = |sum_m w_m A_m(0)|^2 over placed (and docked) models
cudaError_t launch_origin_models(cudaStream_t s, bool fp64, const ModelDev* d_models, int n_models, double* d_res);
cudaError_t launch_pack_values_f32(cudaStream_t s, const float4* grid, int64_t P, double* out);
cudaError_t launch_pack_values_f64(cudaStream_t s, const double4_32a* grid, int64_t P, double* out);
cudaError_t launch_unpack_f64(cudaStream_t s, const double* vals, const double* ders, int64_t P, double4_32a* grid);
cudaError_t launch_unpack_f32(cudaStream_t s, const double* vals, const double* ders, int64_t P, float4* grid);
cudaError_t launch_pack_ders_f32(cudaStream_t s, const float4* grid, int64_t P, double* out);
cudaError_t launch_pack_ders_f64(cudaStream_t s, const double4_32a* grid, int64_t P, double* out);

}  // namespace dpx
