/*
 * oracle.h — CPU restatement of D+'s scattering hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.  The
 * product path (libdpx) never links, loads or calls it.
 *
 * Every function restates an algorithm of the reference (uri-raviv-lab/dplus-dev)
 * and cites the file:line it follows.  Two precisions exist:
 *   ORC_FP64     every float of the reference promoted to double (the parity
 *                target of the GPU paths);
 *   ORC_REFEXACT float where the reference computes in float (phases, sin/cos,
 *                per-atom sums, form factors, spline diagonal), used to time
 *                the reference's CPU algorithm and to measure its own error.
 *
 * Parity pins: the restatement is checked against the reference's golden
 * single-atom fixtures (tests/golden/) and, in the build container, against
 * the reference's own Grid.cpp / Atomic Form Factor.cpp compiled from source
 * into oracle/_ref (see oracle/ref_driver.cpp).
 */
#ifndef DPX_ORACLE_H
#define DPX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_FP64 = 0, ORC_REFEXACT = 1 };

/* form-factor flags, same bit meaning as the reference's atomicFormDefines.h:5-9 */
enum { ORC_CALC_ATOMIC_FORMFACTORS = 1, ORC_CALC_DUMMY_SOLVENT = 2 };

/* ---- grid geometry (Grid.cpp:169-200, 1078-1111) ---- */
int64_t orc_grid_cells(int grid_size);               /* P = 6 L'(L'+1)^2 + 1, L' = grid_size/2 + 3 */
int64_t orc_index_from_indices(int qi, int64_t ti, int64_t pi);
void    orc_indices_from_index(int64_t index, int* qi, int64_t* ti, int64_t* pi);

/* ---- form factors (Atomic Form Factor.cpp:11-27, 91-115, 121-176) ----
 * coeffs: [9 x U] "ion-major" rows (a1,b1,a2,b2,a3,b3,a4,b4,c) as the
 * reference's sortedCoeffs (coeffs[u + k*U]).  ion_rads: [U] nm.
 * out: [nq x U] (q-major), q = q0 + k*dq.  mode: ORC_FP64 / ORC_REFEXACT. */
void orc_aff_table(int U, const double* coeffs, const int* atoms_per_ion,
                   const double* ion_rads, int flags, double sol_ed, double c1,
                   int nq, double q0, double dq, int mode, double* out);

/* ---- amplitude grid fill (Grid.cpp:760-826 + PDBAmplitude.cpp:243-317) ----
 * xyz: [3N] atom coordinates (nm) sorted by ion; data: [2P] interleaved complex. */
void orc_grid_fill(int grid_size, double qmax, int64_t N, const double* xyz,
                   int U, const int* atoms_per_ion, const double* coeffs,
                   const double* ion_rads, int flags, double sol_ed, double c1,
                   double scale, int mode, int nthreads, double* data);

/* Fill only shells [shell_lo, shell_hi] (for bounded CPU-baseline samples). */
void orc_grid_fill_shells(int grid_size, double qmax, int64_t N, const double* xyz,
                          int U, const int* atoms_per_ion, const double* coeffs,
                          const double* ion_rads, int flags, double sol_ed, double c1,
                          double scale, int mode, int nthreads, int shell_lo, int shell_hi,
                          double* data);

/* ---- periodic phi splines (Grid.cpp:1113-1151, PeriodicSplineSolver.h:7-67) ---- */
/* Voxelized-solvent boxes {cx, cy, cz, w, Lx, Ly, Lz, 0} added to every cell
 * (PDBAmplitude.cpp:277-314), times scale. */
void orc_grid_add_boxes(int grid_size, double qmax, int64_t n_boxes, const float* boxes, double scale, int mode,
                        int nthreads, double* data);
/* The same over shells [shell_lo, shell_hi] only. */
void orc_grid_add_boxes_shells(int grid_size, double qmax, int64_t n_boxes, const float* boxes, double scale,
                               int mode, int nthreads, int shell_lo, int shell_hi, double* data);
void orc_grid_splines(int grid_size, const double* data, double* coeffs, int mode, int nthreads);

/* ---- interpolation (Grid.cpp:61-134, 487-607, 677-721) ----
 * amplitude at |q| = qs[k], direction (theta, phi); out: [2 nq] */
void orc_grid_amplitudes_at_points(int grid_size, double qmax, const double* data,
                                   const double* coeffs, int nq, const double* qs,
                                   double theta, double phi, double* out);

/* ---- seeded direction streams ----
 * The reference draws u2, v2 ~ U[0,2) from std::mt19937 (Amplitude.cpp:2764-2780):
 * phi = pi*u2, theta = acos(v2-1).  Writes D pairs (theta, phi). */
void orc_mc_directions(uint32_t seed, int64_t D, double* theta_phi);
/* Per-layer seeds as DomainModel::CalculateIntensityVector + IntegrateLayersTogether
 * derive them (Amplitude.cpp:762-767, 1171-1173) from an injected master seed. */
void orc_layer_seeds(uint32_t master, int nq, int n_layers, uint32_t* seeds);

/* ---- orientation average over one or more leaves ----
 * A "model" here is the reference DomainModel holding leaves; each leaf is a
 * grid with a placement (Euler angles alpha,beta,gamma in radians, translation)
 * and optionally a docked copy list (ManualSymmetry, Symmetries.cpp:1079-1166).
 */
typedef struct orc_leaf {
    const double* data;     /* [2P] */
    const double* coeffs;   /* [2P] */
    double rot[3];          /* leaf orientation (radians), EulerD Amplitude.h:557-573 */
    double tr[3];           /* leaf translation (nm) */
    int    n_copies;        /* 0: plain leaf; >0: docked copies below (ManualSymmetry) */
    const double* copy_rot; /* [3 n_copies] radians (alpha,beta,gamma) */
    const double* copy_tr;  /* [3 n_copies] nm */
    double sym_scale;       /* ManualSymmetry scale */
} orc_leaf;

/* IntegrateLayersTogether + AverageIntensitiesBetweenLayers (Amplitude.cpp:1168-1247,
 * 2746-2822).  dirs: theta/phi pairs; layer l uses dirs + 2*l*dir_layer_stride
 * (stride 0 = one shared set).  max_iter samples at most; eps > 0 enables the
 * reference's 4-point history convergence test every 100 samples. */
int orc_integrate_layers(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves,
                         int nq, const double* Q, const double* dirs, int64_t dir_layer_stride,
                         int64_t max_iter, double eps, int nthreads, double* res);

/* The same with the reference GPU averages' convergence test (GPUCalcMCOAJacobSphrDD,
 * OAJacob.cu:244-346; GPUHybridCalc.cu:467-578, 705-720): with eps > 0 the running
 * mean after every samples_per_step samples, converged from the 4th step on when
 * every q of the bracket is within eps of its mean at each of the 3 steps before. */
int orc_integrate_layers_gpu_rule(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, int nq,
                                  const double* Q, const double* dirs, int64_t dir_layer_stride, int64_t max_iter,
                                  double eps, int64_t samples_per_step, int nthreads, double* res);

/* Bracket assignment of IntegrateLayersTogether (Amplitude.cpp:1184-1217):
 * for each q index, the layer whose bracket computes it (-1 for q == 0), later
 * layers win where two brackets claim the same q. */
void orc_q_brackets(int grid_size, double qmax, int nq, const double* Q, int* layer_of_q);

/* ---- VEGAS (restated from the reference's GPU-only implementation,
 * HybridOA.cu:182-501 and GPUHybridCalc.cu:326-333, 363-375, 581-720) ----
 * 32 x 32 bins over (u, v) in [0,1)^2 with theta = acos(1 - 2u), phi = 2 pi v;
 * points_per_iter points per iteration (a multiple of 1024), uniforms from the
 * counter-based stream orc_uniform(seed, (bracket << 32) | iteration, n); the
 * bin grid carries over from bracket to bracket, as in the reference.
 * Brackets follow the hybrid path's rule (GPUHybridCalc.cu:363-375). */
double orc_uniform(uint64_t seed, uint64_t key, uint64_t n);
int orc_vegas_intensity(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, int nq, const double* Q,
                        uint64_t seed, int points_per_iter, int64_t max_points, double eps, double* res);

/* ---- grid-path assembly: out[cell] += scale * lattice(q) * sum_leaves amplitude(q)
 * through GetCart, as Grid::Fill evaluates ManualSymmetry / GridSymmetry
 * calcAmplitude (Symmetries.cpp:105-137, 697-716, 879-962).  lattice: NULL or
 * {a[3], b[3], c[3], Na, Nb, Nc}. */
void orc_assemble_grid(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, const double* lattice,
                       double scale, int nthreads, double* out);

/* ---- FP64 direct-sum oracle (no grid) ----
 * F(q n) = scale [sum_j f_j(q) e^{i q n.r_j} + sum_b w_b prod_a L_a sinc(q_a L_a/2)
 * e^{i q n.c_b}] for a leaf (PDBAmplitude::calcAmplitude, PDBAmplitude.cpp:243-317,
 * every float promoted to double) with optional voxelized-solvent boxes
 * {cx, cy, cz, w, Lx, Ly, Lz, 0} and docked copies (sum_c e^{i q n.t_c}
 * F(R_c^T q n), Symmetries.cpp:1079-1166); I(q) = mean over the given
 * directions of |F|^2. */
void orc_direct_intensity(int64_t N, const double* xyz, int U, const int* atoms_per_ion,
                          const double* coeffs, const double* ion_rads, int flags,
                          double sol_ed, double c1, double scale, int64_t n_boxes, const float* boxes,
                          int n_copies, const double* copy_rot, const double* copy_tr,
                          int nq, const double* Q, int64_t D, const double* dirs,
                          int nthreads, double* res);

/* ---- adaptive Gauss-Kronrod 7/15 (Amplitude.cpp:1416-1467, mathfuncs.h:104-124) ----
 * integrand = |sum of leaves|^2 through the grid (GetCart path). */
double orc_gk_intensity(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves,
                        double q, double eps, int64_t max_depth);

/* ---- Debye sum (DebyeCalTester::Calculate, PDBAmplitude.cpp:1789-1825) ----
 * xyz [3N] nm sorted by ion; bfactor [N] (Debye-Waller) and anom [2N]
 * (f', f'') per atom or NULL; out [nq].  mode ORC_FP64 / ORC_REFEXACT. */
void orc_debye(int64_t N, const double* xyz, int U, const int* atoms_per_ion, const double* coeffs,
               const double* ion_rads, int flags, double sol_ed, double c1, const double* bfactor,
               const double* anom, int nq, const double* Q, int mode, int nthreads, double* out);

/* ---- synthetic workload structures (shared by the CPU baseline and the tests) ----
 * Seeded globule: a self-avoiding walk of 0.15 nm steps folded into a sphere of
 * radius_nm, elements C 63 / N 17 / O 19 / S 1 % (codes 0..3); the generator of
 * the library's dpx_make_globule.  Returns 0, or -1 when the sphere cannot hold
 * the atoms. */
int orc_make_globule(int64_t n_atoms, double radius_nm, uint64_t seed, float* xyz, int* elem);

#ifdef __cplusplus
}
#endif
#endif
