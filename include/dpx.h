/*
 * dpx.h — C-ABI of the GB300-native D+ scattering hot path (libdpx.so).
 *
 * Plain pointers, sizes and status codes; no C++ or torch types cross this
 * boundary, and no entry point throws, traps or falls back to the CPU.  Every
 * entry point returns DPX_OK (0) or a negative dpx_status; the message of the
 * last failure on the calling thread is dpx_last_error().
 *
 * Reference interfaces replaced (uri-raviv-lab/dplus-dev):
 *   dpx_pdb_jacobian_grid_amplitude  <- PDBJacobianGridAmplitudeCalculation
 *                                       (Backend/Backend/PDBAmplitudeCUDA.h:7-13,
 *                                        impl PDBAmplitudeCUDA.cu:442-458)
 *   dpx_calc_mcoa_jacob_sphr         <- GPUCalcMCOAJacobSphrDD
 *                                       (Backend/GPU/GPUHeader.h:236, OAJacob.cu:387-399)
 *   dpx_grid_compute_splines         <- JacobianSphereGrid::CalculateSplines
 *                                       (Backend/Backend/Grid.cpp:1113-1151)
 *   dpx_grid_fill_pdb                <- PDBAmplitude::calculateGrid GPU branch
 *                                       (Backend/Backend/PDBAmplitude.cpp:319-435)
 *   dpx_orientation_average          <- DomainModel::IntegrateLayersTogether /
 *                                       AverageIntensitiesBetweenLayers
 *                                       (Backend/Backend/Amplitude.cpp:1168-1247, 2746-2822)
 *                                       and the hybrid ManualSymmetry docked sum
 *                                       (Backend/DefaultModels/Symmetries.cpp:1079-1166,
 *                                        GPUHybridCalc.cu:467-578)
 *   dpx_calc_man_sym_jacob_sphr      <- GPUCalcManSymJacobSphrDD (Backend/GPU/GPUHeader.h:185)
 *   dpx_calc_spc_fill_sym_jacob_sphr <- GPUCalcSpcFillSymJacobSphrDD (GPUHeader.h:214)
 *   dpx_sum_grids_jacob_sphr         <- GPUSumGridsJacobSphrDD (GPUHeader.h:255)
 *   dpx_mc_directions / dpx_layer_seeds <- the mt19937 draws of
 *                                       Amplitude.cpp:757-767, 1171-1173, 2764-2780
 *   dpx_debye_intensity              <- DebyeCalTester::Calculate / CalculateVectorGPU
 *                                       (Backend/Backend/PDBAmplitude.cpp:1652-1716, 1789-1967)
 *   dpx_calc_debye_v2                <- GPUCalcDebyeV2 (Backend/GPU/InternalGPUHeaders.h:61,
 *                                       DebyeCalculator.cu:164-372)
 *   dpx_pdb_jacobian_grid_amplitude_aff <- PDBJacobianGridAmplitudeCalculation with the
 *                                       form factors as its atomicFFCalculator tabulates them
 *                                       (PDBAmplitudeCUDA.cu:224-284)
 *   dpx_hybrid_*                     <- IGPUGridCalculator of GPUCreateCalculatorHybrid
 *                                       (Backend/GPU/GPUInterface.h:203-222, GPUHeader.cpp:39-42)
 *                                       and GPUHybrid_SetPDB / GPUHybrid_PDBAmplitude
 *                                       (HybridPDB.cu:168-379)
 */
#ifndef DPX_H
#define DPX_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum dpx_status {
    DPX_OK = 0,
    DPX_ERR_ARG = -1,       /* invalid argument / inconsistent sizes */
    DPX_ERR_CUDA = -2,      /* CUDA runtime error (message in dpx_last_error) */
    DPX_ERR_OOM = -3,       /* device allocation failed */
    DPX_ERR_STOPPED = -4,   /* *pStop was set by the caller */
    DPX_ERR_NODEVICE = -5   /* no CUDA device */
} dpx_status;

typedef enum dpx_precision {
    DPX_FP64 = 0,   /* plain FP64: FP64 phases, sincos, accumulation, FP64 grid */
    DPX_FP32 = 1    /* FP32 bulk: FP32 phases/SFU sincos/accumulation, FP32 grid,
                       FP64 centring and translation phases, FP64 reductions */
} dpx_precision;

/* form-factor flags (same bits as the reference's atomicFormDefines.h:5-9) */
#define DPX_CALC_ATOMIC_FORMFACTORS 1
#define DPX_CALC_DUMMY_SOLVENT 2

typedef struct dpx_ctx_s* dpx_ctx;
typedef struct dpx_grid_s* dpx_grid;

const char* dpx_last_error(void);
int dpx_version(void);

/* ---- context: one device, one stream, grow-only device scratch ---- */
int dpx_ctx_create(int device, dpx_ctx* out);
int dpx_ctx_destroy(dpx_ctx ctx);
/* Use an external cudaStream_t (NULL = the context's own stream).  The
 * harmonic fill also runs its radial tables and its atoms' moments on a second
 * stream the context owns, forked from and joined back into this one by
 * events; the fill returns with both drained. */
int dpx_ctx_set_stream(dpx_ctx ctx, void* stream);
void* dpx_ctx_get_stream(dpx_ctx ctx);
int dpx_ctx_synchronize(dpx_ctx ctx);
/* FP32 amplitude-kernel launch shape: phi cells per work item x threads per
 * block (the threads also set the atoms per shared-memory tile), chosen by
 * dpx_autotune_fill (default 8 x 128, flat).  Supported: 2x256, 4x128, 4x256,
 * 6x128, 6x256, 8x128, 8x256. */
int dpx_ctx_set_fill_shape(dpx_ctx ctx, int cells_per_thread, int threads);
/* FP32 fill schedule: 0 = flat (one CTA per tile of THREADS work items, the
 * hardware hands them out), 1 = persistent (one CTA per resident slot pulling
 * tiles from an atomic counter). */
int dpx_ctx_set_fill_schedule(dpx_ctx ctx, int persistent);
/* Phi columns per work item whose sin/cos run as polynomials on the FMA pipe
 * instead of the SFU (0-3 for the 8 x 128 shape, 0 otherwise; reset to 0 by
 * dpx_ctx_set_fill_shape): meant to share the work between the two pipes; on
 * GB300 they measure slower than the SFU alone and the autotuner keeps 0. */
int dpx_ctx_set_fill_poly(dpx_ctx ctx, int poly_columns);
/* FP32 fill method.  DPX_FILL_DIRECT: the direct sum over points and cells
 * (the reference's algorithm, PDBAmplitude.cpp:243-317).  DPX_FILL_HARMONIC
 * (the default; no counterpart in the reference): the same amplitudes by
 * multipole expansion.  Per shell i the plane-wave expansion is cut at order
 * l_i = ceil(q_i R + 3 (q_i R)^(1/3) + 6) (R the largest point distance from
 * the centre); points are grouped by radius and their expansion coefficients
 * summed per group, a group of radial bin b to the order its largest radius
 * needs (the same rule at q_max); each theta row is synthesized from the
 * coefficients; solvent
 * boxes are expanded into their voxels (dpx_pdb_desc.voxel_step).  It serves
 * dpx_grid_fill_pdb and dpx_grid_fill_pdb_batch; leaves it cannot take (boxes
 * without a voxel step, orders above 175, more than 1024 radial bins of
 * solvent) use the direct sum, as do FP64 grids and the batched-solve and
 * serving fills.  dpx_autotune_fill times it beside the direct shapes (the
 * row {0, 0, 0, 0} of dpx_fill_shapes). */
enum { DPX_FILL_DIRECT = 0, DPX_FILL_HARMONIC = 1 };
/* Directions per thread (1, the default, or 2) of the FP32 orientation average
 * of one undocked leaf over a shared direction set, for every context of the
 * process: 2 gives each thread the samples of two neighbouring chunks, twice
 * the independent gathers in flight at a higher register count. */
int dpx_set_average_shape(int directions_per_thread);
/* Moments kernel of the harmonic fill, for every context of the process (no
 * counterpart in the reference): DPX_MOMENTS_MMA_F16 (the default) computes the
 * moments with the warp-level mma.sync path, FP16 operands split into value and
 * remainder (m16n8k16); DPX_MOMENTS_MMA_SYNC the same with TF32 split operands
 * (m16n8k8: twice the MMAs); DPX_MOMENTS_TCGEN05 on the fifth-generation tensor
 * cores (tcgen05.mma with FP16 split operands, accumulators in tensor memory).
 * All three give the same amplitudes within the FP32 bound.  Harmonic plans
 * made after the call use it (prepared leaves and batches keep the kernel they
 * were planned with). */
enum { DPX_MOMENTS_TCGEN05 = 0, DPX_MOMENTS_MMA_SYNC = 1, DPX_MOMENTS_MMA_F16 = 2 };
int dpx_set_moments_kernel(int kind);
int dpx_get_moments_kernel(void);
/* Faults recorded by this library's kernels on the current device since the
 * last call (no counterpart in the reference): *flags = 0 when there were none;
 * bits 0-3: a wait of the tensor-core moments kernel ran past its limit (that
 * kernel then leaves its moments unwritten and returns).  Reads and clears the
 * flags; synchronous. */
int dpx_take_device_faults(unsigned* flags);
int dpx_ctx_set_fill_method(dpx_ctx ctx, int method);
int dpx_ctx_get_fill_method(dpx_ctx ctx);
/* Convergence test of the Monte Carlo average (eps > 0) for this context's
 * dpx_orientation_average calls.  DPX_CONV_CPU (the default): the reference's
 * CPU rule (DomainModel::AverageIntensitiesBetweenLayers, Backend/Backend/
 * Amplitude.cpp:2773-2815): every 100th sample from the 400th on, each q's
 * running mean within eps of the 4 last recorded.  DPX_CONV_GPU: the rule of
 * the reference's GPU averages (GPUCalcMCOAJacobSphrDD, Backend/GPU/OAJacob.cu:
 * 244-346, 8192 samples a step; the hybrid GPUHybridCalculator::
 * MonteCarloOrientationFunc, GPUHybridCalc.cu:467-578 with checkConvergenceOA
 * :705-720, 4096 a step): the running mean after every samples_per_step
 * samples (a multiple of 128); from the 4th step on, converged when every q of
 * the bracket is within eps of its mean at each of the 3 steps before. */
enum { DPX_CONV_CPU = 0, DPX_CONV_GPU = 1 };
int dpx_ctx_set_convergence(dpx_ctx ctx, int rule, int64_t samples_per_step);
/* Stage timing of harmonic fills (no counterpart in the reference): with
 * timing on, the fill records CUDA events on the context's stream;
 * dpx_ctx_stage_times then gives out[5] = {ms of the moments kernels, ms of
 * the synthesis, ms of the whole harmonic fill, points (atoms + voxels), the
 * mean over the points of the (l, m) moments each one carries (its radial
 * bin's (l_b + 1)(l_b + 2) / 2)} of the last harmonic fill (zeros when there
 * was none). */
int dpx_ctx_set_timing(dpx_ctx ctx, int on);
int dpx_ctx_stage_times(dpx_ctx ctx, double* out);
/* With timing on: *ms = the device time of the last dpx_orientation_average's
 * main kernel alone (CUDA events around that launch; 0 when there was none). */
int dpx_ctx_average_kernel_ms(dpx_ctx ctx, double* ms);
/* shape[4] = {cells_per_thread, threads, persistent, poly_columns} in use. */
int dpx_ctx_get_fill_shape(dpx_ctx ctx, int* shape);
/* The shapes the autotuner sweeps: writes 4 ints per shape (if shapes != NULL)
 * and returns their number. */
int dpx_fill_shapes(int* shapes);

/* ---- grid geometry (Grid.cpp:169-200): P = 6 L'(L'+1)^2 + 1, L' = grid_size/2 + 3 ---- */
int64_t dpx_grid_cells(int grid_size);
int64_t dpx_grid_bytes(int grid_size, int precision);

/* ---- device-resident JacobianSphereGrid (values + phi-spline derivatives) ---- */
int dpx_grid_create(dpx_ctx ctx, int grid_size, double qmax, int precision, dpx_grid* out);
int dpx_grid_destroy(dpx_grid g);
void* dpx_grid_device_ptr(dpx_grid g);     /* float4 / double4 {re, im, dre, dim} per cell */
int dpx_grid_info(dpx_grid g, int* grid_size, double* qmax, int* precision, int64_t* cells);

/* Amplitude of a PDB leaf on every cell (atoms + Gaussian dummy-atom solvent):
 *   F(q) = scale * sum_u aff_u(|q|) sum_{j in u} e^{i q.r_j}
 * atoms: float4 (x, y, z, ignored) in nm, sorted by ion; host or device memory.
 * coeffs: [9 x n_ions], coeffs[u + k*n_ions] = (a1,b1,a2,b2,a3,b3,a4,b4,c)[k]
 * (the reference's sortedCoeffs layout); ion_rads: [n_ions] dummy-atom radii (nm).
 * center: optional [3] centring translation c restored as a per-cell phase
 * e^{i q.c}.  Host atoms are shifted by c here (NULL: their centroid for FP32
 * grids, 0 for FP64 grids); device atoms are taken as already shifted by the
 * caller (r_device = r - c; NULL: c = 0). */
int dpx_grid_fill_pdb(dpx_grid g, int64_t n_atoms, const float* atoms, int atoms_on_device, int n_ions,
                      const int* atoms_per_ion, const double* coeffs, const double* ion_rads, int flags,
                      double solvent_ed, double c1, double scale, const double* center);
/* One PDB leaf of a batched fill: the arguments of dpx_grid_fill_pdb after the grid. */
typedef struct dpx_pdb_desc {
    int64_t n_atoms;
    const float* atoms;
    int atoms_on_device;
    int n_ions;
    const int* atoms_per_ion;
    const double* coeffs;
    const double* ion_rads;
    int flags;
    double solvent_ed;
    double c1;
    double scale;
    const double* center;
    /* voxelized solvent (dpx_voxel_solvent), 0 / NULL for none: n_boxes
     * records of 8 floats {cx, cy, cz, weight (e/nm^3), Lx, Ly, Lz, 0} in nm,
     * in the frame of the host atoms; each adds
     * weight * prod_a [L_a sinc(q_a L_a / 2)] e^{i q.c} (PDBAmplitude.cpp:277-314)
     * before the scale. */
    int64_t n_boxes;
    const float* boxes;
    /* the voxel edge (nm) the boxes were built on; 0 = unknown.  The
     * harmonic fill expands boxes into voxels and needs it. */
    double voxel_step;
    /* optional: the ions' form factors already tabulated on the grid's
     * shells, as the reference's atomicFFCalculator::GetQMajorAFFMatrix(aff,
     * aff_n, step) writes them (Backend/GPU/Atomic Form Factor.cpp:58-64, called
     * so by PDBAmplitudeCUDA.cu:284): aff[u * aff_n + k] at q = k * step, the
     * dummy-atom solvent included, aff_n >= the grid's layers + 4.  When set,
     * coeffs, ion_rads, flags, solvent_ed and c1 are not read; the FP64 direct
     * sum and the Debye sum, which need form factors at any q, reject such a
     * leaf.  NULL: the form factors are computed from the coefficients. */
    const float* aff;
    int aff_n;
} dpx_pdb_desc;
/* Fills n grids (distinct, one context) from n leaves.  The FP32 grids of the
 * batch share ONE launch over the tiles of every leaf (flat: one CTA per tile;
 * or persistent, dpx_ctx_set_fill_schedule), so small leaves no longer leave
 * SMs idle; FP64 grids get a launch each.  Same results as n calls of dpx_grid_fill_pdb.  The reference
 * fills each PDBAmplitude in its own call (Amplitude.cpp PDBAmplitude::calculateGrid). */
int dpx_grid_fill_pdb_batch(int n, const dpx_grid* grids, const dpx_pdb_desc* pdbs);
/* Autotuner (no counterpart in the reference): fills the batch once per shape
 * of dpx_fill_shapes (after one warm-up fill), times the FP32 fill launch with
 * CUDA events, averages over `repeats`, and keeps the fastest shape in the
 * context.  best[4] (optional) receives it, times_ms[dpx_fill_shapes()]
 * (optional) the average time of each.  The grids end up filled. */
int dpx_autotune_fill(int n, const dpx_grid* grids, const dpx_pdb_desc* pdbs, int repeats, int* best,
                      float* times_ms);
/* ---- prepared leaves (the reference's PDBAmplitude after PreCalculate,
 * Backend/Backend/PDBAmplitude.cpp:1199-1336: what does not change between
 * fills, done once) ----
 * dpx_leaf_create prepares the fill of grid g from leaf d (host or device atoms,
 * as dpx_grid_fill_pdb_batch reads them; host arrays are read only here): for
 * an FP32 grid with the harmonic method, the harmonic fill's plan (points
 * grouped by radius and ion, solvent boxes expanded and binned on the device,
 * recurrence tables) and its launch scratch, in device memory the leaf owns;
 * otherwise the direct sum's staged tables.  It synchronizes the context's
 * stream.  dpx_leaf_fill queues the fill of g, with its phi-spline derivatives,
 * on the context's stream and returns without waiting: no host work, no copies
 * from the host and no synchronization, so a stream capture can record it.
 * The grid must outlive the leaf.  dpx_leaf_info: harmonic (1) or direct (0),
 * kernel launches per fill, device bytes the leaf holds. */
typedef struct dpx_leaf_s* dpx_leaf;
int dpx_leaf_create(dpx_grid g, const dpx_pdb_desc* d, dpx_leaf* out);
int dpx_leaf_fill(dpx_leaf leaf);
int dpx_leaf_info(dpx_leaf leaf, int* harmonic, int64_t* launches, int64_t* device_bytes);
int dpx_leaf_destroy(dpx_leaf leaf);
/* Periodic cubic-spline phi derivatives of every theta row. */
int dpx_grid_compute_splines(dpx_grid g);
/* Host copies in the reference's layout: interleaved complex double [2P] each;
 * either pointer may be NULL. */
int dpx_grid_read(dpx_grid g, double* values, double* coeffs);
int dpx_grid_write(dpx_grid g, const double* values, const double* coeffs);

/* ---- orientation average ----
 * A model is a leaf grid placed by Euler angles rot[3] (radians, Tait-Bryan
 * X1Y2Z3 as EulerD) and a translation tr[3] (nm), optionally docked n_copies
 * times (ManualSymmetry rows: copy_rot[3 n] radians, copy_tr[3 n] nm, scale
 * sym_scale).  All models share grid_size and qmax.
 * Q: [nq] ascending q (nm^-1).  Directions: (theta, phi) pairs; layer l uses
 * dirs + 2*l*dir_layer_stride (0 = one shared set); dirs_on_device selects
 * host or device memory.  n_samples per bracket; eps > 0 applies the
 * reference's convergence test every 100 samples.  res: [nq] host. */
int dpx_orientation_average(dpx_ctx ctx, int n_models, const dpx_grid* grids, const double* rot,
                            const double* tr, const int* n_copies, const double* copy_rot,
                            const double* copy_tr, const double* sym_scale, int nq, const double* Q,
                            const double* dirs, int dirs_on_device, int64_t dir_layer_stride,
                            int64_t n_samples, double eps, double* res);

/* VEGAS orientation average (the reference's GPU-only method,
 * HybridOA.cu:182-501 / GPUHybridCalc.cu:581-720, driven by
 * DomainModel::CalculateIntensityVector, Amplitude.cpp:737-754): 32 x 32 bins over
 * (u, v), theta = acos(1 - 2u), phi = 2 pi v; points_per_iter points per
 * iteration (a multiple of 1024; the reference uses 4096), iterations until
 * max_points or the reference's 3-iteration convergence test at eps; the bin
 * grid carries over between brackets as in the reference.  Uniforms come from
 * a counter-based stream keyed by (seed, bracket, iteration), so results are
 * reproducible.  Model arguments as dpx_orientation_average. */
int dpx_vegas_intensity(dpx_ctx ctx, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                        const int* n_copies, const double* copy_rot, const double* copy_tr, const double* sym_scale,
                        int nq, const double* Q, uint64_t seed, int points_per_iter, int64_t max_points, double eps,
                        double* res);

/* Grid-path assembly: dst[cell] += scale * lattice(q) * sum of the placed (and
 * docked) source grids at the cell's q, through the single-q GetCart path.
 * Replaces ManualSymmetry::calculateGrid / GPUCalcManSymJacobSphrDD
 * (Symmetries.cpp:879-962, GPUHeader.h:185, ManSymGenJacob.cu:36-124), the
 * grid sum GPUSumGridsJacobSphrDD (GPUHeader.h:255, SumGridsJacobian.cu:44-130)
 * and the space-filling GridSymmetry (Symmetries.cpp:60-137,
 * GPUCalcSpcFillSymJacobSphrDD, GPUHeader.h:214): lattice = NULL or the 12
 * doubles {a[3], b[3], c[3], Na, Nb, Nc} giving sum_n e^{i n q.a} per axis.
 * The destination accumulates, as the reference's outputs do; compute its
 * splines afterwards.  Sources share the destination's size, qmax, precision. */
int dpx_grid_assemble(dpx_grid dst, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                      const int* n_copies, const double* copy_rot, const double* copy_tr, const double* sym_scale,
                      const double* lattice, double scale);

/* Adaptive Gauss-Kronrod (7,15) orientation average (DomainModel::
 * GaussKron2DSphereRecurs / GaussLegTheta / GaussLegPhi, Amplitude.cpp:1416-1467,
 * CPU-only in the reference): theta in [0, pi/2], phi in [0, 2 pi], bisection
 * until |1 - G7/K15| <= eps or the depth budget max_depth (the reference's
 * "iterations") is spent, result / 2 pi.  The recursion runs on the host; each
 * level's phi intervals are evaluated in one batched launch through the single-q
 * GetSphr interpolation.  Q need not be sorted.  Model arguments as
 * dpx_orientation_average. */
int dpx_gk_intensity(dpx_ctx ctx, int n_models, const dpx_grid* grids, const double* rot, const double* tr,
                     const int* n_copies, const double* copy_rot, const double* copy_tr, const double* sym_scale,
                     int nq, const double* Q, double eps, int64_t max_depth, double* res);

/* ---- seeded direction streams (product-side restatement of the reference's draws) ---- */
/* D pairs (theta, phi) from std::mt19937(seed) with u2, v2 ~ U[0,2): phi = pi u2, theta = acos(v2 - 1) */
int dpx_mc_directions(uint32_t seed, int64_t D, double* theta_phi);
/* Per-layer seeds derived from a master seed the way CalculateIntensityVector
 * and IntegrateLayersTogether draw them (nq draws discarded, then n_layers+1). */
int dpx_layer_seeds(uint32_t master, int nq, int n_layers, uint32_t* seeds);
/* Which layer's bracket computes each q (-1 for q == 0), as IntegrateLayersTogether. */
int dpx_q_brackets(int grid_size, double qmax, int nq, const double* Q, int* layer_of_q);

/* ---- synthetic structures ----
 * Seeded self-avoiding random walk (0.15 nm steps) folded into a sphere of
 * radius_nm; elements drawn C 63 % / N 17 % / O 19 % / S 1 % (codes 0..3). */
int dpx_make_globule(int64_t n_atoms, double radius_nm, uint64_t seed, float* xyz, int* elem);

/* ---- drop-in replacements with the reference's argument meaning ---- */
/* PDBJacobianGridAmplitudeCalculation: outData is a caller-owned host buffer of
 * 2*voxels doubles in grid-index order; splines are left to the caller, as in
 * the reference.  Voxelized solvent as the reference passes it: solCOM /
 * outSolCOM float4 box centres (nm), solDims / outSolDims int4 extents in
 * voxels of voxStep nm; excluded-volume boxes count at -solventED when
 * bitCombination has CALC_VOXELIZED_SOLVENT (1 << 3), solvation boxes at
 * outerSolED - solventED, each set only with more than four boxes.  Returns 0
 * or a negative status (the reference returns -3000-err / -1000-err; callers
 * test != 0). */
/* The same with the form factors as the reference's call site has them: affs
 * [numUniqueIons][nq] from atomicFFCalculator::GetQMajorAFFMatrix(affs, nq,
 * stepSize) with nq = the grid's layers + 4 (numQLayers + 1 of
 * PDBAmplitudeCUDA.cu:224-284), the dummy-atom solvent folded in; atomsPerIon
 * from GetNumAtomsPerIon; bitCombination from GetBitCombination (its
 * CALC_VOXELIZED_SOLVENT bit selects the excluded-volume boxes). */
int dpx_pdb_jacobian_grid_amplitude_aff(uint64_t voxels, int thDivs, int phDivs, double stepSize, double* outData,
                                        const float* atomLocations, int64_t numAtoms, int numUniqueIons,
                                        const int* atomsPerIon, const float* affs, int nq, int bitCombination,
                                        float solventED, const float* solCOM, const int* solDims, int64_t nSol,
                                        double voxStep, const float* outSolCOM, const int* outSolDims,
                                        int64_t nOutSol, double outerSolED, double scale, int precision, int* pStop);
int dpx_pdb_jacobian_grid_amplitude(uint64_t voxels, int thDivs, int phDivs, double stepSize, double* outData,
                                    const float* atomLocations, int64_t numAtoms, int numUniqueIons,
                                    const int* atomsPerIon, const float* coeffs, const float* ionRads,
                                    int bitCombination, float solventED, float c1, const float* solCOM,
                                    const int* solDims, int64_t nSol, double voxStep, const float* outSolCOM,
                                    const int* outSolDims, int64_t nOutSol, double outerSolED, double scale,
                                    int precision, int* pStop);
/* GPUCalcMCOAJacobSphrDD with explicit directions: inAmp / inD are the grid's
 * values and spline derivatives [2 voxels]; intensities [qPoints]. */
int dpx_calc_mcoa_jacob_sphr(int64_t voxels, int thDivs, int phDivs, double stepSz, const double* inAmp,
                             const double* inD, const double* qs, double* intensities, int qPoints,
                             int64_t maxIters, double convergence, const double* dirs, int64_t dir_layer_stride,
                             int precision, int* pStop);
/* ---- Debye sum: the exact orientation average of a PDB leaf, no grid ----
 *   I(q) = scale^2 [sum_i |f_i|^2 + 2 sum_{i<j} Re(f_i conj f_j) sin(q r_ij)/(q r_ij)]
 * (DebyeCalTester::Calculate, PDBAmplitude.cpp:1789-1825; AnomDebyeCalTester,
 * :2466-2512).  f_i is the ion's form factor minus its Gaussian dummy-atom
 * solvent (d->flags, solvent_ed, c1, ion_rads as for the grid fill), plus
 * anomalous[2i] + i anomalous[2i+1] (f', f'') when anomalous != NULL, times
 * exp(-bfactors[i] (q/10)^2 / (16 pi^2)) when bfactors != NULL; per-atom
 * arrays follow d->atoms' (ion-sorted) order.  d must carry no voxel boxes.
 * Q, I: host [nq].  FP32: FP32 pair terms (SFU sine, Taylor series below
 * q r = 0.5), FP64 per-tile and cross-block sums; FP64: every step in double.
 * Device scratch: (nq x N x 4 B, twice with anomalous factors, FP64: 8 B)
 * on the context, kept for reuse. */
int dpx_debye_intensity(dpx_ctx ctx, const dpx_pdb_desc* d, const float* bfactors, const float* anomalous, int nq,
                        const double* Q, int precision, double* I);
/* GPUCalcDebyeV2 (DebyeCalculator.cu:350-372): numQValues q values
 * qMin + k (qMax - qMin) / (numQValues - 1) (in float, as the reference);
 * loc: float4 [numAtoms] nm sorted by ion; atomsPerIon read up to numAtoms;
 * coeffs [9 x U]; anomalousVals: float2 [numAtoms] or NULL; dummy-atom solvent
 * (bSol, solvED != 0) with ion radii atmRad[atmInd[first atom of the ion]];
 * bSolOnly drops the atomic form factors; ionInd is unused (as in the
 * reference).  B factors are applied when bBfactors is set, as the reference's
 * CPU Debye does (its GPU kernel ignores them).  outData [numQValues]. */
int dpx_calc_debye_v2(int numQValues, float qMin, float qMax, double* outData, int numAtoms, const int* atomsPerIon,
                      const float* loc, const unsigned char* ionInd, const float* anomalousVals, int bBfactors,
                      const float* BFactors, const float* coeffs, int bSol, int bSolOnly, const char* atmInd,
                      const float* atmRad, float solvED, float c1, int precision, int* pStop);
/* GPUCalcManSymJacobSphrDD (Backend/GPU/GPUHeader.h:185, ManSymGenJacob.cu:36-124,
 * called by ManualSymmetry::calculateGrid Symmetries.cpp:943-945).  loc*
 * arrays hold numCopies + 1 entries: entry 0 places the inner object, entries
 * 1..numCopies are the copies (nm, radians).  outData [2 voxels] is
 * accumulated: outData += scale * sum_k R_k A(R_k^T q) e^{i q.t_k}. */
int dpx_calc_man_sym_jacob_sphr(int64_t voxels, int thDivs, int phDivs, int numCopies, double stepSize,
                                const double* inModel, double* outData, const double* ds, const double* locX,
                                const double* locY, const double* locZ, const double* locA, const double* locB,
                                const double* locC, double scale, int precision, int* pStop);
/* GPUCalcSpcFillSymJacobSphrDD (GPUHeader.h:214, SymmetryGenJacob.cu:33-140):
 * vectorMatrix [9] = the three unit-cell vectors a, b, c (nm), repeats [3],
 * innerRots [3] (radians), innerTrans [3] (nm); outData is accumulated with
 * the kernel's lattice sum  sum_{n<N} e^{-i n q.a}  per vector. */
int dpx_calc_spc_fill_sym_jacob_sphr(int64_t voxels, int thDivs, int phDivs, double stepSize, const double* inModel,
                                     double* outData, const double* ds, const double* vectorMatrix,
                                     const double* repeats, const double* innerRots, const double* innerTrans,
                                     double scale, int precision, int* pStop);
/* GPUSumGridsJacobSphrDD (GPUHeader.h:255, SumGridsJacobian.cu:44-256):
 * outAmpData [2 voxels] = sum over numGrids placed grids (trans [3 n] nm,
 * rots [3 n] radians); the output is overwritten, as in the reference. */
int dpx_sum_grids_jacob_sphr(int64_t voxels, int thDivs, int phDivs, double stepSz, const double* const* inAmpData,
                             const double* const* inD, const double* trans, const double* rots, int numGrids,
                             double* outAmpData, int precision, int* pStop);

/* ---- FP64 direct-sum orientation average: the error reference of every grid
 * result (no counterpart as one call in the reference; it evaluates
 * PDBAmplitude::calcAmplitude, Backend/Backend/PDBAmplitude.cpp:243-317, with
 * its solvent boxes :277-314, point by point in FP64, with no grid) ----
 *   I(q_k) = (1/D) sum_d |F(q_k n_d)|^2,
 *   F(q) = scale [sum_u aff_u(|q|) sum_{j in u} e^{i q.r_j}
 *                 + sum_b w_b prod_a L_a sinc(q_a L_a / 2) e^{i q.c_b}]
 * for the leaf d (host atoms and boxes, in the frame given: no centring), or
 * with n_copies > 0 the docked sum sum_c e^{i q.t_c} F(R_c^T q) (copy_rot
 * [3 n] radians as EulerD, copy_tr [3 n] nm; ManualSymmetry, Symmetries.cpp:
 * 1079-1166).  Q [nq] any order; dirs [D] (theta, phi) pairs, host; res [nq]
 * host.  FP64 throughout, deterministic (fixed-order sums); cost N x nq x D
 * FP64 sincos, so callers use it on a sample of q values and directions. */
int dpx_direct_intensity(dpx_ctx ctx, const dpx_pdb_desc* d, int n_copies, const double* copy_rot,
                         const double* copy_tr, int nq, const double* Q, int64_t D, const double* dirs, double* res);

/* ---- the hybrid calculator: IGPUGridCalculator (Backend/GPU/GPUInterface.h:
 * 203-222) made by GPUCreateCalculatorHybrid (GPUHeader.cpp:39-42) and driven by
 * DomainModel::PerformGPUHybridComputation (Backend/Backend/Amplitude.cpp:
 * 2044-2289), with its leaf hooks GPUHybrid_SetPDB / GPUHybrid_PDBAmplitude
 * (HybridPDB.cu:168-379) and GPUHybrid_AmpGridAmplitude ----
 * dpx_hybrid_create = GPUCreateCalculatorHybrid + Initialize of the master
 * workspace: the q points as the reference passes them (float, ascending,
 * within qMax), totalSize = 2 x cells, thetaDivisions 3, phiDivisions 6,
 * qLayers = layers + 4, qMax, stepSize; FP32 bulk or plain FP64 grids.
 * A child is one distinct leaf: its amplitude grid comes from a PDB leaf (the
 * fill of dpx_grid_fill_pdb_batch, with its phi-spline derivatives) or from
 * given amplitudes [2 cells] (derivatives computed).  AddRotations gives a
 * child's rotations as float4 {alpha, beta, gamma (radians, EulerD), scale}
 * and AddTranslations, per rotation index, its translations as float4
 * {x, y, z (nm), 0} (the flattened tree, Amplitude.cpp:2151-2183).
 * ComputeIntensity: I(q) = < |sum_children sum_rotations scale sum_translations
 * e^{i q.t} A_child(R^T q)|^2 > over orientations, outData [nq]:
 *   DPX_OA_MC     seeded mt19937 directions (min(iterations, 2^22) of them,
 *                 shared by the brackets) and the reference GPU averages'
 *                 convergence test at epsi, 4096 samples a step
 *                 (GPUHybridCalc.cu:467-578, 705-720);
 *   DPX_OA_VEGAS  dpx_vegas_intensity with 4096 points an iteration up to
 *                 iterations points (GPUHybridCalc.cu:581-703).
 * pStop is read before and after.  dpx_hybrid_destroy = FreeWorkspace + delete. */
enum { DPX_OA_MC = 0, DPX_OA_VEGAS = 1 };
typedef struct dpx_hybrid_s* dpx_hybrid;
int dpx_hybrid_create(dpx_ctx ctx, int nq, const float* qPoints, int64_t totalSize, int thetaDivs, int phiDivs,
                      int qLayers, double qMax, double stepSize, int precision, dpx_hybrid* out);
int dpx_hybrid_set_num_children(dpx_hybrid h, int n);
int dpx_hybrid_child_pdb(dpx_hybrid h, int child, const dpx_pdb_desc* d);
int dpx_hybrid_child_amp(dpx_hybrid h, int child, const double* amp);
int dpx_hybrid_add_rotations(dpx_hybrid h, int child, int n, const float* rotations);
int dpx_hybrid_add_translations(dpx_hybrid h, int child, int rotation, int n, const float* translations);
int dpx_hybrid_compute_intensity(dpx_hybrid h, int method, double* outData, double epsi, int64_t iterations,
                                 uint64_t seed, int* pStop);
int dpx_hybrid_destroy(dpx_hybrid h);

/* SFU calibration (no counterpart in the reference): times a kernel of
 * independent __sincosf chains and returns the MUFU operations per second this
 * GPU sustains (sin and cos count one each) — the denominator of the amplitude
 * fill's roofline. */
int dpx_measure_sfu_peak(dpx_ctx ctx, double* ops_per_s);
/* Pipe calibration (no counterpart in the reference): flops_per_s[4] = the
 * FP32 FMA pipe with scalar FMAs, with packed f32x2 FMAs, the TF32 mma.sync
 * (m16n8k8) and the FP16 mma.sync (m16n8k16, FP32 accumulators) tensor paths
 * this GPU sustains, each from a kernel of independent chains — the
 * denominators of the harmonic moments' roofline. */
int dpx_measure_pipe_peaks(dpx_ctx ctx, double* flops_per_s);
/* tcgen05 issue calibration (no counterpart in the reference): one thread
 * issues 32 MMAs of kind::f16, M = 128 (A in tensor memory, B in shared
 * memory) into one accumulator; cycles_per_mma[2] = SM cycles per MMA from the
 * first issue to the commit's completion at N = 16 and at N = 256 — the
 * evidence for which shapes the fifth-generation tensor cores can be fed at. */
int dpx_measure_tcgen05_issue(dpx_ctx ctx, double* cycles_per_mma);

/* ---- amplitude-grid files (D+'s binary .amp, version 13: JacobianSphereGrid::
 * ExportBinaryData / ImportBinaryData, Backend/Backend/Grid.cpp:847-963) ----
 * values: 2 * dpx_grid_cells(grid_size) doubles, the interleaved complex
 * amplitudes in grid-index order (dpx_grid_read / dpx_grid_write layout);
 * step = qmax / (grid_size / 2).  Host file I/O; spline coefficients are not
 * stored (a reader recomputes them, as D+ does). */
int dpx_amp_write(const char* path, const char* header, int grid_size, double step, const double* values);
/* grid_size, step and the header text (NUL-terminated, truncated to header_cap). */
int dpx_amp_read_info(const char* path, int* grid_size, double* step, char* header, int64_t header_cap);
int dpx_amp_read(const char* path, double* values);

/* ---- voxelized solvent (PDBAmplitude::FindPDBRanges PDBAmplitude.cpp:710-749,
 * CalculateSolventSpace VoxelizedSolvent.cpp:4-190) ----
 * Voxelizes the space around n_atoms atoms (xyz: 3 floats per atom, nm;
 * radii: per atom, nm — the radius table of the leaf's radius type) with
 * voxel_step, marks the excluded volume, a probe shell (probe_radius) and the
 * solvation layer (solvation_thickness), optionally fills enclosed cavities,
 * and reduces both regions to boxes in the reference's greedy scan order.
 * Box set 0 = excluded volume, 1 = solvation layer: centres (3 floats, nm)
 * and extents in voxels (3 ints).  Host computation. */
typedef struct dpx_boxes_s* dpx_boxes;
int dpx_voxel_solvent(int64_t n_atoms, const float* xyz, const float* radii, double voxel_step, double probe_radius,
                      double solvation_thickness, int fill_holes, dpx_boxes* out);
int64_t dpx_boxes_count(dpx_boxes b, int which);
int dpx_boxes_get(dpx_boxes b, int which, float* com, int* dims);
/* dims[3] = the voxel space (x, y, z padded to a multiple of 16) */
int dpx_boxes_space(dpx_boxes b, int64_t* dims);
int dpx_boxes_free(dpx_boxes b);

/* ---- batched independent solves (no counterpart in the reference, which
 * solves one structure per call) ----
 * Each solve is one PDB leaf on its own grid (grid_size, qmax) with its own
 * ascending q list: fill -> splines -> Monte Carlo average over the shared
 * direction set (n_samples (theta, phi) pairs, host), eps as in
 * dpx_orientation_average.  dpx_batch_create uploads every input once, packs
 * the solves in order into waves whose grids fit grid_budget_bytes (<= 0: half
 * the free device memory) and records one CUDA graph per wave: one FP32 fill
 * launch over the wave's structures (FP64: one per structure), then splines,
 * average, finalize and the q = 0 term per structure, then one copy of the
 * wave's I(q) to pinned host memory.  Host atoms are read only during create;
 * device atoms (atoms_on_device) must stay valid while the batch lives. */
typedef struct dpx_solve_desc {
    dpx_pdb_desc pdb;
    int grid_size;
    double qmax;
    int nq;
    const double* Q;
} dpx_solve_desc;
typedef struct dpx_batch_s* dpx_batch;
int dpx_batch_create(dpx_ctx ctx, int n, const dpx_solve_desc* solves, int precision, const double* dirs,
                     int64_t n_samples, double eps, int64_t grid_budget_bytes, dpx_batch* out);
/* Launch every wave's graph on the context stream (returns at once) / and wait. */
int dpx_batch_launch(dpx_batch b);
int dpx_batch_run(dpx_batch b);
/* I(q) of solve j after a completed run: res [nq of solve j]. */
int dpx_batch_result(dpx_batch b, int j, double* res);
/* Waves, kernel launches per run, bytes of the grid pool. */
int dpx_batch_info(dpx_batch b, int* n_waves, int64_t* kernels_per_run, int64_t* pool_bytes);
int dpx_batch_destroy(dpx_batch b);

/* ---- serving engine (no counterpart in the reference, which runs one job
 * at a time on its job thread, JobManager.cpp:151-206) ----
 * A request is an I(q) solve of placed, optionally docked PDB leaves on one
 * grid (grid_size, qmax, precision): models name a leaf, a placement (rot,
 * tr: [3 n_models] radians / nm, NULL = identity) and optional copies as in
 * dpx_orientation_average.  Inputs are copied at submission.  One worker
 * thread admits requests in arrival order while the device-memory budget
 * holds (grids not yet resident + scratch; unpinned cached grids are evicted
 * least-recently-used first; a request that does not fit yet lets later
 * ones pass), fills all grids the admitted requests miss in one batched
 * launch, and runs each request's Monte Carlo average on one of n_streams
 * streams, so requests that arrive while others run overlap with them.  Grids
 * stay resident keyed by leaf content (or leaf_keys[l] != 0) and grid
 * parameters: requests that change only placements reuse them.  The shared
 * direction set (n_dirs (theta, phi) pairs) is given once; a request uses its
 * first n_samples. */
typedef struct dpx_request {
    int n_leaves;
    const dpx_pdb_desc* leaves;   /* host atoms */
    const uint64_t* leaf_keys;    /* NULL or per leaf; 0 = key by content */
    int n_models;
    const int* model_leaf;        /* [n_models] leaf index per model */
    const double* rot;
    const double* tr;
    const int* n_copies;          /* NULL = no docked copies */
    const double* copy_rot;
    const double* copy_tr;
    const double* sym_scale;      /* NULL = 1 */
    int grid_size;
    double qmax;
    int precision;
    int nq;
    const double* Q;              /* ascending, within [0, qmax] */
    int64_t n_samples;
    double eps;
} dpx_request;
typedef struct dpx_server_stats {
    int64_t submitted, completed, failed;
    int64_t grid_fills;           /* leaves filled */
    int64_t grid_hits;            /* leaves found resident */
    int64_t fill_launches, steps, evictions;
    int64_t bytes_in_use, bytes_peak, budget;
    int64_t cached_grids;
} dpx_server_stats;
typedef struct dpx_server_s* dpx_server;
/* hbm_budget_bytes <= 0: 80% of the free device memory. */
int dpx_server_create(dpx_ctx ctx, int64_t hbm_budget_bytes, int max_inflight, int n_streams, const double* dirs,
                      int64_t n_dirs, dpx_server* out);
int dpx_server_submit(dpx_server s, const dpx_request* r, uint64_t* ticket);
/* 1 when the request has finished (or failed), 0 while it waits or runs. */
int dpx_server_poll(dpx_server s, uint64_t ticket);
/* Blocks until the request finishes; res [nq]; latency_ms = submission to
 * completion.  Returns the request's status; the ticket is then released. */
int dpx_server_wait(dpx_server s, uint64_t ticket, double* res, double* latency_ms);
int dpx_server_stats_get(dpx_server s, dpx_server_stats* st);
/* Finishes every submitted request, then frees the server. */
int dpx_server_destroy(dpx_server s);

/* ---- allocation-free orientation average ----
 * No counterpart in the reference.  For callers that cannot call cudaMalloc /
 * cudaFree: applications whose device memory is pre-reserved by their own pool
 * or caching allocator, and latency-bound serving loops in which a cudaFree
 * (which synchronizes the whole device) would stall other streams.
 *
 * The Monte Carlo orientation average of one device-resident grid at identity
 * placement (the computation of dpx_calc_mcoa_jacob_sphr / GPUCalcMCOAJacobSphrDD
 * on device data).  The caller passes every input and output:
 *   grid_cells  device cells of the grid (dpx_grid_device_ptr layout: float4 for
 *               DPX_FP32, 32-byte double4 for DPX_FP64, values + spline derivatives)
 *   Q           host, nq ascending q values within the grid's qmax
 *   dirs        device, n_samples (theta, phi) pairs used by every layer bracket
 *   res         device, nq doubles, written in full
 *   stream      cudaStream_t the work is queued on (NULL = legacy default stream);
 *               the call returns without waiting for the results.
 * Nothing is allocated on the device: bracket tables and partial sums live in
 * one static scratch array of DPX_NOALLOC_SCRATCH_BYTES compiled into libdpx,
 * which every GPU that loads the library holds until the process exits.
 * Requests needing more (about 8 B x brackets x ceil(n_samples/128) x max q per
 * bracket) return DPX_ERR_ARG.  The first call on a device looks up the scratch
 * array's device address (cudaGetSymbolAddress) with that device current; make
 * that first call before any stream capture.  The address is kept per device
 * ordinal, i.e. for the CUDA runtime's primary context of that device: callers
 * that switch the thread to another driver-API context of the same device must
 * not use this entry point there.  All calls on a device share the
 * array and it keeps the last call's contents: calls whose work overlaps on the
 * GPU (different streams, or different host threads) race on it and must be
 * serialized by the caller. */
#define DPX_NOALLOC_SCRATCH_BYTES (16u << 20)
int dpx_mc_average_noalloc(const void* grid_cells, int grid_size, double qmax, int precision, int nq,
                           const double* Q, const double* dirs, int64_t n_samples, double eps, double* res,
                           void* stream);

#ifdef __cplusplus
}
#endif
#endif
