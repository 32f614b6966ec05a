// dplus_gpu_shims.cpp — the reference-side binding of libdpx.
//
// D+'s GPU entry points with their own signatures, forwarding to libdpx's
// C-ABI (include/dpx.h).  A D+ maintainer compiles this file into D+'s backend
// in place of the CUDA sources that define the same functions
// (Backend/Backend/PDBAmplitudeCUDA.cu, Backend/GPU/OAJacob.cu,
// ManSymGenJacob.cu, SymmetryGenJacob.cu, SumGridsJacobian.cu, GPUHeader.cpp's
// hybrid factory and HybridPDB.cu's leaf hooks) and links -ldpx; the call sites
// (PDBAmplitude.cpp, Amplitude.cpp, Symmetries.cpp) compile unchanged.  Built
// against D+'s own headers: -I Common -I Backend -I Backend/Backend
// -I Backend/GPU and CUDA's include directory for vector_types.h.
//
// Every function returns the reference's success value (0, or true) on
// DPX_OK and its failure value otherwise, so the callers' existing fallbacks
// (e.g. PDBAmplitude.cpp:425-429 to the CPU) take over; the message is
// dpx_last_error().
#include "GPUInterface.h"
#include "PDBAmplitudeCUDA.h"  // PDBJacobianGridAmplitudeCalculation, atomicFFCalculator

#include "dpx.h"

#include <cstdint>
#include <ctime>
#include <map>
#include <mutex>
#include <vector>

namespace {

// Shells of a Jacobian sphere grid of `voxels` cells: L' + 1 (numQLayers + 1
// of PDBAmplitudeCUDA.cu:224-227), or 0 when the count is not such a grid.
int shells_of(long long voxels) {
    for (long long lp = 4; lp < 4096; ++lp) {
        const long long P = 6 * lp * (lp + 1) * (lp + 1) + 1;
        if (P == voxels) return (int)lp + 1;
        if (P > voxels) break;
    }
    return 0;
}

void voxel_arrays(const std::vector<float4>& com, const std::vector<int4>& dims, const float** c, const int** d,
                  int64_t* n) {
    *c = com.empty() ? nullptr : reinterpret_cast<const float*>(com.data());
    *d = dims.empty() ? nullptr : reinterpret_cast<const int*>(dims.data());
    *n = (int64_t)dims.size();
}

}  // namespace

// ---- 1. grid fill: PDBAmplitude::calculateGrid's GPU branch (PDBAmplitude.cpp:417-423) ----
int PDBJacobianGridAmplitudeCalculation(u64 voxels, int thDivs, int phDivs, float stepSize, double* outData,
                                        std::vector<float4> atomLocations, atomicFFCalculator& affCalculator,
                                        std::vector<float4> solCOM, std::vector<int4> solDims, float solvED,
                                        double voxStep, std::vector<float4> outSolCOM, std::vector<int4> outSolDims,
                                        double outerSolED, double scale, progressFunc progfunc, void* progargs,
                                        float progmin, float progmax, int* pStop) {
    const int nq = shells_of((long long)voxels);
    const int U = affCalculator.GetNumUniqueIon();
    if (nq <= 0 || U <= 0) return -1000 - DPX_ERR_ARG;
    // the form factors exactly as the reference's own GPU fill tabulates them
    // (PDBAmplitudeCUDA.cu:284): [U][nq], the dummy-atom solvent included
    std::vector<float> affs((size_t)U * nq);
    affCalculator.GetQMajorAFFMatrix(affs.data(), nq, stepSize);
    std::vector<int> api(U);
    for (int u = 0; u < U; ++u) api[u] = affCalculator.GetNumAtomsPerIon(u);
    const float *sc, *oc;
    const int *sd, *od;
    int64_t ns, no;
    voxel_arrays(solCOM, solDims, &sc, &sd, &ns);
    voxel_arrays(outSolCOM, outSolDims, &oc, &od, &no);
    if (progfunc) progfunc(progargs, progmin);
    const int rc = dpx_pdb_jacobian_grid_amplitude_aff(
        voxels, thDivs, phDivs, stepSize, outData, reinterpret_cast<const float*>(atomLocations.data()),
        (int64_t)atomLocations.size(), U, api.data(), affs.data(), nq, affCalculator.GetBitCombination(), solvED,
        sc, sd, ns, voxStep, oc, od, no, outerSolED, scale, DPX_FP32, pStop);
    if (progfunc) progfunc(progargs, progmax);
    return rc == DPX_OK ? 0 : -1000 + rc;
}

int PDBJacobianGridAmplitudeCalculation(u64 voxels, int thDivs, int phDivs, float stepSize, float* outData,
                                        std::vector<float4> atomLocations, atomicFFCalculator& affCalculator,
                                        std::vector<float4> solCOM, std::vector<int4> solDims, float solvED,
                                        double voxStep, std::vector<float4> outSolCOM, std::vector<int4> outSolDims,
                                        double outerSolED, double scale, progressFunc progfunc, void* progargs,
                                        float progmin, float progmax, int* pStop) {
    std::vector<double> d(2 * (size_t)voxels);
    const int rc = PDBJacobianGridAmplitudeCalculation(voxels, thDivs, phDivs, stepSize, d.data(), atomLocations,
                                                       affCalculator, solCOM, solDims, solvED, voxStep, outSolCOM,
                                                       outSolDims, outerSolED, scale, progfunc, progargs, progmin,
                                                       progmax, pStop);
    if (rc == 0)
        for (size_t i = 0; i < d.size(); ++i) outData[i] = (float)d[i];
    return rc;
}

// ---- 2. grid Monte Carlo orientation average (GPUHeader.h:236, OAJacob.cu:387-399) ----
int GPUCalcMCOAJacobSphrDD(long long voxels, int thDivs, int phDivs, double stepSz, double* inAmpData, double* inD,
                           double* qs, double* intensities, int qPoints, long long maxIters, double convergence,
                           progressFunc progfunc, void* progargs, float progmin, float progmax, int* pStop) {
    const int shells = shells_of(voxels);
    if (shells <= 0) return -1000 - DPX_ERR_ARG;
    const int L = shells - 4;  // the radial layers: gridSize / 2
    // the reference draws its directions from a clock-seeded mt19937
    // (OAJacob.cu:221-222); libdpx takes them as input: one set per layer,
    // drawn in the reference's order from seeds derived as Amplitude.cpp:1171-1173
    std::vector<uint32_t> seeds(L + 1);
    dpx_layer_seeds((uint32_t)std::time(nullptr), qPoints, L, seeds.data());
    std::vector<double> dirs(2 * (size_t)L * (size_t)maxIters);
    for (int l = 0; l < L; ++l) dpx_mc_directions(seeds[l], maxIters, dirs.data() + 2 * (size_t)l * maxIters);
    if (progfunc) progfunc(progargs, progmin);
    const int rc = dpx_calc_mcoa_jacob_sphr(voxels, thDivs, phDivs, stepSz, inAmpData, inD, qs, intensities, qPoints,
                                            maxIters, convergence, dirs.data(), maxIters, DPX_FP64, pStop);
    if (progfunc) progfunc(progargs, progmax);
    return rc == DPX_OK ? 0 : -3000 + rc;
}

// ---- 3. assembly grids (GPUHeader.h:185, 214, 255) ----
int GPUCalcManSymJacobSphrDD(long long voxels, int thDivs, int phDivs, int numCopies, double stepSize,
                             double* inModel, double* outData, double* ds, double* locX, double* locY, double* locZ,
                             double* locA, double* locB, double* locC, double scale, progressFunc, void*, float,
                             float, int* pStop) {
    const int rc = dpx_calc_man_sym_jacob_sphr(voxels, thDivs, phDivs, numCopies, stepSize, inModel, outData, ds,
                                               locX, locY, locZ, locA, locB, locC, scale, DPX_FP64, pStop);
    return rc == DPX_OK ? 0 : -3000 + rc;
}

int GPUCalcSpcFillSymJacobSphrDD(long long voxels, int thDivs, int phDivs, double stepSize, double* inModel,
                                 double* outData, double* ds, double* vectorMatrix, double* repeats, double* innerRots,
                                 double* innerTrans, double scale, progressFunc, void*, float, float, int* pStop) {
    const int rc = dpx_calc_spc_fill_sym_jacob_sphr(voxels, thDivs, phDivs, stepSize, inModel, outData, ds,
                                                    vectorMatrix, repeats, innerRots, innerTrans, scale, DPX_FP64,
                                                    pStop);
    return rc == DPX_OK ? 0 : -3000 + rc;
}

int GPUSumGridsJacobSphrDD(long long voxels, int thDivs, int phDivs, double stepSz, double** inAmpData, double** inD,
                           double* trans, double* rots, int numGrids, double* outAmpData, progressFunc, void*, float,
                           float, int* pStop) {
    const int rc = dpx_sum_grids_jacob_sphr(voxels, thDivs, phDivs, stepSz, inAmpData, inD, trans, rots, numGrids,
                                            outAmpData, DPX_FP64, pStop);
    return rc == DPX_OK ? 0 : -3000 + rc;
}

// ---- 4. the hybrid calculator (GPUInterface.h:203-222, GPUHeader.cpp:39-42) ----
namespace {

// GPUHybrid_SetPDB's inputs of a child, kept until GPUHybrid_PDBAmplitude fills it.
struct PendingPDB {
    std::vector<float> atoms;   // float4 per atom
    std::vector<float> affs;    // [U][qLayers]
    std::vector<int> api;
    std::vector<float> boxes;   // 8 per box {cx, cy, cz, w, Lx, Ly, Lz, 0}
    double voxStep = 0;
    double scale = 1;
    int qLayers = 0;
};
std::mutex g_mu;
std::map<const GridWorkspace*, PendingPDB> g_pending;

class DpxHybridCalculator : public IGPUGridCalculator {
public:
    // IGPUGridCalculator has no virtual destructor, so the caller's delete
    // (Amplitude.cpp:2284) does not reach this class: the master workspace's
    // FreeWorkspace releases libdpx's objects.

    // Called for the master workspace, then for each child (Amplitude.cpp:2180-2189).
    bool Initialize(int gpuID, const std::vector<float>& qPoints, long long totalSize, int thetaDivisions,
                    int phiDivisions, int qLayers, double qMax, double stepSize, GridWorkspace& res) override {
        res.calculator = this;
        res.gpuID = gpuID;
        res.totalsz = totalSize;
        res.thetaDivs = thetaDivisions;
        res.phiDivs = phiDivisions;
        res.qLayers = qLayers;
        res.qMax = (float)qMax;
        res.stepSize = (float)stepSize;
        if (h_) return true;  // a child: the master made the calculator
        if (dpx_ctx_create(gpuID, &ctx_) != DPX_OK) return false;
        return dpx_hybrid_create(ctx_, (int)qPoints.size(), qPoints.data(), totalSize, thetaDivisions, phiDivisions,
                                 qLayers, qMax, stepSize, DPX_FP32, &h_) == DPX_OK;
    }

    bool SetNumChildren(GridWorkspace& workspace, int numChildren) override {
        workspace.children = new GridWorkspace[numChildren];
        workspace.numChildren = numChildren;
        for (int c = 0; c < numChildren; ++c) {
            workspace.children[c].parent = &workspace;
            workspace.children[c].calculator = this;
        }
        return h_ && dpx_hybrid_set_num_children(h_, numChildren) == DPX_OK;
    }

    bool AddRotations(GridWorkspace& workspace, std::vector<float4>& rotations) override {
        return h_ && dpx_hybrid_add_rotations(h_, child_index(workspace), (int)rotations.size(),
                                              reinterpret_cast<const float*>(rotations.data())) == DPX_OK;
    }

    bool AddTranslations(GridWorkspace& workspace, int rotationIndex, std::vector<float4>& translations) override {
        return h_ && dpx_hybrid_add_translations(h_, child_index(workspace), rotationIndex, (int)translations.size(),
                                                 reinterpret_cast<const float*>(translations.data())) == DPX_OK;
    }

    bool ComputeIntensity(std::vector<GridWorkspace>& workspaces, double* outData, double epsi, long long iterations,
                          progressFunc progfunc, void* progargs, float progmin, float progmax, int* pStop) override {
        if (!h_ || workspaces.empty()) return false;
        const int method = workspaces[0].intMethod == OA_ADAPTIVE_MC_VEGAS ? DPX_OA_VEGAS : DPX_OA_MC;
        if (progfunc) progfunc(progargs, progmin);
        // the reference seeds its device generator from the clock (GPUHybridCalc.cu:196-198)
        const int rc = dpx_hybrid_compute_intensity(h_, method, outData, epsi, iterations,
                                                    (uint64_t)std::time(nullptr), pStop);
        if (progfunc) progfunc(progargs, progmax);
        return rc == DPX_OK;
    }

    bool FreeWorkspace(GridWorkspace& workspace) override {
        if (!workspace.parent) {  // the master: the calculator's libdpx objects go with it
            if (h_) dpx_hybrid_destroy(h_);
            if (ctx_) dpx_ctx_destroy(ctx_);
            h_ = nullptr;
            ctx_ = nullptr;
        }
        if (workspace.children) {
            std::lock_guard<std::mutex> lock(g_mu);
            for (int c = 0; c < workspace.numChildren; ++c) g_pending.erase(&workspace.children[c]);
            delete[] workspace.children;
            workspace.children = nullptr;
            workspace.numChildren = 0;
        }
        return true;
    }

    dpx_hybrid handle() const { return h_; }

    static int child_index(const GridWorkspace& w) {
        return w.parent && w.parent->children ? (int)(&w - w.parent->children) : -1;
    }

private:
    dpx_ctx ctx_ = nullptr;
    dpx_hybrid h_ = nullptr;
};

DpxHybridCalculator* calculator_of(GridWorkspace& work) { return dynamic_cast<DpxHybridCalculator*>(work.calculator); }

}  // namespace

IGPUGridCalculator* GPUCreateCalculatorHybrid() { return new DpxHybridCalculator(); }

// PDBAmplitude::SetModel's hook (PDBAmplitude.cpp:1417-1452): the leaf's atoms,
// form factors as its atomicFFCalculator tabulates them on the workspace's
// shells, and voxelized solvent, selected as HybridPDB.cu:355-356 does.
bool GPUHybrid_SetPDB(GridWorkspace& work, const std::vector<float4>& atomLocs,
                      const std::vector<float>& atomicFormFactors_q_major_ordering, double solventRad,
                      float4* solCOM, int4* solDims, int solDimLen, float voxStep, float4* outSolCOM,
                      int4* outSolDims, int outSolDimLen, float outerSolED) {
    PendingPDB p;
    p.atoms.assign(reinterpret_cast<const float*>(atomLocs.data()),
                   reinterpret_cast<const float*>(atomLocs.data()) + 4 * atomLocs.size());
    p.affs = atomicFormFactors_q_major_ordering;
    p.api.assign(work.atomsPerIon, work.atomsPerIon + work.numUniqueIons);
    p.voxStep = voxStep;
    p.scale = work.scale;
    p.qLayers = work.qLayers;
    auto add = [&](const float4* com, const int4* dims, int n, double w) {
        for (int b = 0; b < n; ++b) {
            const float rec[8] = {com[b].x, com[b].y, com[b].z, (float)w, voxStep * (float)dims[b].x,
                                  voxStep * (float)dims[b].y, voxStep * (float)dims[b].z, 0.f};
            p.boxes.insert(p.boxes.end(), rec, rec + 8);
        }
    };
    if (work.solventED != 0.0f && work.solventType != 4 && work.solventType > 0)
        add(solCOM, solDims, solDimLen, -work.solventED);
    if (work.solventED != outerSolED && outerSolED != 0.0f && solventRad > 0.0)
        add(outSolCOM, outSolDims, outSolDimLen, outerSolED - work.solventED);
    std::lock_guard<std::mutex> lock(g_mu);
    g_pending[&work] = std::move(p);
    return true;
}

bool GPUHybrid_PDBAmplitudeDLL(GridWorkspace& work) {
    DpxHybridCalculator* calc = calculator_of(work);
    PendingPDB p;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_pending.find(&work);
        if (!calc || it == g_pending.end()) return false;
        p = std::move(it->second);
        g_pending.erase(it);
    }
    const int U = (int)p.api.size();
    dpx_pdb_desc d{};
    d.n_atoms = (int64_t)p.atoms.size() / 4;
    d.atoms = p.atoms.data();
    d.n_ions = U;
    d.atoms_per_ion = p.api.data();
    d.scale = p.scale;
    d.n_boxes = (int64_t)p.boxes.size() / 8;
    d.boxes = p.boxes.empty() ? nullptr : p.boxes.data();
    d.voxel_step = p.voxStep;
    d.aff = p.affs.data();
    d.aff_n = p.qLayers;
    return dpx_hybrid_child_pdb(calc->handle(), DpxHybridCalculator::child_index(work), &d) == DPX_OK;
}

// AmpGridAmplitude's hook: a given amplitude grid (values, interleaved complex).
bool GPUHybrid_AmpGridAmplitudeDLL(GridWorkspace& work, double* amp) {
    DpxHybridCalculator* calc = calculator_of(work);
    return calc && dpx_hybrid_child_amp(calc->handle(), DpxHybridCalculator::child_index(work), amp) == DPX_OK;
}
