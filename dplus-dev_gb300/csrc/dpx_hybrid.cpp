// dpx_hybrid.cpp — the reference's hybrid GPU calculator behind a C-ABI.
//
// D+ computes a model tree that does not use grids all the way up with its
// hybrid calculator (IGPUGridCalculator, Backend/GPU/GPUInterface.h:203-222,
// made by GPUCreateCalculatorHybrid, GPUHeader.cpp:39-42, driven by
// DomainModel::PerformGPUHybridComputation, Amplitude.cpp:2044-2289): every
// distinct leaf gets an amplitude grid (GPUHybrid_SetPDB / GPUHybrid_PDBAmplitude,
// HybridPDB.cu:168-379, or a given amplitude grid), the flattened tree gives each
// leaf a list of rotations {alpha, beta, gamma, scale} and per rotation a list
// of translations, and ComputeIntensity averages |sum over leaves, rotations and
// translations of e^{i q.t} A_leaf(R^T q)|^2 over orientations by Monte Carlo
// or VEGAS, bracket by bracket.
//
// Here a leaf is a device-resident grid (harmonic or direct fill, or written),
// and each (leaf, rotation scale) becomes one docked model of
// dpx_orientation_average / dpx_vegas_intensity: its rotations repeated over
// their translations as copies, grouped by rotation on the device.  Monte Carlo
// runs with the reference GPU averages' convergence test (4096 samples a step).
#include "dpx_host.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <vector>

using namespace dpxh;

namespace {
struct HybridChild {
    dpx_grid grid = nullptr;
    std::vector<std::array<float, 4>> rots;                  // {alpha, beta, gamma, scale}
    std::vector<std::vector<std::array<float, 4>>> trans;    // per rotation {x, y, z, 0}
};
}  // namespace

struct dpx_hybrid_s {
    dpx_ctx ctx = nullptr;
    int grid_size = 0;
    double qmax = 0.0;
    int precision = DPX_FP32;
    std::vector<double> Q;
    std::vector<HybridChild> children;
};

namespace {
void hybrid_free(dpx_hybrid h) {
    for (HybridChild& c : h->children)
        if (c.grid) dpx_grid_destroy(c.grid);
    ctx_release(h->ctx);
    delete h;
}

int child_of(dpx_hybrid h, int child, HybridChild** out) {
    if (!h) return fail(DPX_ERR_ARG, "hybrid calculator is NULL");
    if (child < 0 || child >= (int)h->children.size())
        return fail(DPX_ERR_ARG, "child %d of %zu (SetNumChildren first)", child, h->children.size());
    *out = &h->children[child];
    return DPX_OK;
}

int new_grid(dpx_hybrid h, HybridChild& c) {
    if (c.grid) {
        dpx_grid_destroy(c.grid);
        c.grid = nullptr;
    }
    return dpx_grid_create(h->ctx, h->grid_size, h->qmax, h->precision, &c.grid);
}
}  // namespace

extern "C" {

int dpx_hybrid_create(dpx_ctx ctx, int nq, const float* qPoints, int64_t totalSize, int thetaDivs, int phiDivs,
                      int qLayers, double qMax, double stepSize, int precision, dpx_hybrid* out) {
    if (!ctx || !qPoints || nq <= 0 || !out) return fail(DPX_ERR_ARG, "NULL or empty argument");
    if (precision != DPX_FP32 && precision != DPX_FP64) return fail(DPX_ERR_ARG, "bad precision");
    *out = nullptr;
    if (totalSize <= 0 || (totalSize & 1)) return fail(DPX_ERR_ARG, "totalSize must be twice the cells");
    int grid_size = 0;
    double qmax = 0.0;
    if (int rc = grid_from_voxels(totalSize / 2, thetaDivs, phiDivs, stepSize, &grid_size, &qmax)) return rc;
    if (qLayers != grid_size / 2 + 4)
        return fail(DPX_ERR_ARG, "qLayers=%d; a grid of %lld cells has %d", qLayers, (long long)(totalSize / 2),
                    grid_size / 2 + 4);
    if (std::fabs(qmax - qMax) > 1e-6 * std::max(1.0, qMax))
        return fail(DPX_ERR_ARG, "qMax=%g does not match stepSize x layers = %g", qMax, qmax);
    std::vector<double> Q(qPoints, qPoints + nq);
    for (int k = 0; k < nq; ++k) {
        if (!(Q[k] >= 0.0) || Q[k] > qmax * (1.0 + 1e-6))
            return fail(DPX_ERR_ARG, "q=%g outside [0, qMax]", Q[k]);
        if (k && Q[k] < Q[k - 1]) return fail(DPX_ERR_ARG, "q points must be ascending");
        Q[k] = std::min(Q[k], qmax);
    }
    if (int rc = set_device(ctx)) return rc;
    auto* h = new dpx_hybrid_s;
    h->ctx = ctx;
    ctx_retain(ctx);
    h->grid_size = grid_size;
    h->qmax = qmax;
    h->precision = precision;
    h->Q = std::move(Q);
    *out = h;
    return DPX_OK;
}

int dpx_hybrid_set_num_children(dpx_hybrid h, int n) {
    if (!h || n < 0) return fail(DPX_ERR_ARG, "bad argument");
    for (size_t c = n; c < h->children.size(); ++c)
        if (h->children[c].grid) dpx_grid_destroy(h->children[c].grid);
    h->children.resize(n);
    return DPX_OK;
}

int dpx_hybrid_child_pdb(dpx_hybrid h, int child, const dpx_pdb_desc* d) {
    HybridChild* c = nullptr;
    if (int rc = child_of(h, child, &c)) return rc;
    if (!d) return fail(DPX_ERR_ARG, "NULL leaf");
    if (int rc = new_grid(h, *c)) return rc;
    if (int rc = dpx_grid_fill_pdb_batch(1, &c->grid, d)) return rc;
    return dpx_grid_compute_splines(c->grid);
}

int dpx_hybrid_child_amp(dpx_hybrid h, int child, const double* amp) {
    HybridChild* c = nullptr;
    if (int rc = child_of(h, child, &c)) return rc;
    if (!amp) return fail(DPX_ERR_ARG, "NULL amplitudes");
    if (int rc = new_grid(h, *c)) return rc;
    if (int rc = dpx_grid_write(c->grid, amp, nullptr)) return rc;
    return dpx_grid_compute_splines(c->grid);
}

int dpx_hybrid_add_rotations(dpx_hybrid h, int child, int n, const float* rotations) {
    HybridChild* c = nullptr;
    if (int rc = child_of(h, child, &c)) return rc;
    if (n < 0 || (n > 0 && !rotations)) return fail(DPX_ERR_ARG, "bad rotations");
    for (int r = 0; r < n; ++r) {
        c->rots.push_back({rotations[4 * r], rotations[4 * r + 1], rotations[4 * r + 2], rotations[4 * r + 3]});
        c->trans.emplace_back();
    }
    return DPX_OK;
}

int dpx_hybrid_add_translations(dpx_hybrid h, int child, int rotation, int n, const float* translations) {
    HybridChild* c = nullptr;
    if (int rc = child_of(h, child, &c)) return rc;
    if (rotation < 0 || rotation >= (int)c->rots.size())
        return fail(DPX_ERR_ARG, "rotation %d of %zu", rotation, c->rots.size());
    if (n < 0 || (n > 0 && !translations)) return fail(DPX_ERR_ARG, "bad translations");
    for (int t = 0; t < n; ++t)
        c->trans[rotation].push_back(
            {translations[4 * t], translations[4 * t + 1], translations[4 * t + 2], translations[4 * t + 3]});
    return DPX_OK;
}

int dpx_hybrid_compute_intensity(dpx_hybrid h, int method, double* outData, double epsi, int64_t iterations,
                                 uint64_t seed, int* pStop) {
    if (!h || !outData) return fail(DPX_ERR_ARG, "NULL argument");
    if (method != DPX_OA_MC && method != DPX_OA_VEGAS) return fail(DPX_ERR_ARG, "unknown method %d", method);
    if (iterations <= 0) return fail(DPX_ERR_ARG, "iterations must be positive");
    if (pStop && *pStop) return fail(DPX_ERR_STOPPED, "stopped");
    // one docked model per (leaf, rotation scale): its rotations x their translations
    std::vector<dpx_grid> grids;
    std::vector<double> rot, tr, crot, ctr, sscale;
    std::vector<int> ncop;
    for (HybridChild& c : h->children) {
        if (!c.grid) return fail(DPX_ERR_ARG, "a child has no amplitude grid");
        std::map<float, std::vector<size_t>> by_scale;
        for (size_t r = 0; r < c.rots.size(); ++r) by_scale[c.rots[r][3]].push_back(r);
        for (auto& kv : by_scale) {
            int n = 0;
            for (size_t r : kv.second)
                for (const auto& t : c.trans[r]) {
                    for (int k = 0; k < 3; ++k) crot.push_back((double)c.rots[r][k]);
                    for (int k = 0; k < 3; ++k) ctr.push_back((double)t[k]);
                    ++n;
                }
            if (!n) continue;
            grids.push_back(c.grid);
            for (int k = 0; k < 3; ++k) {
                rot.push_back(0.0);
                tr.push_back(0.0);
            }
            ncop.push_back(n);
            sscale.push_back((double)kv.first);
        }
    }
    if (grids.empty()) return fail(DPX_ERR_ARG, "no rotations and translations were added");
    const int nm = (int)grids.size();
    const int nq = (int)h->Q.size();
    int rc = DPX_OK;
    if (method == DPX_OA_MC) {
        // the reference draws uniforms on the device per step; here a seeded
        // mt19937 set of directions (the reference's draw order), as many as
        // the iterations allow up to 2^22, shared by every bracket
        const int64_t D = std::min<int64_t>(iterations, (int64_t)1 << 22);
        std::vector<double> dirs((size_t)2 * D);
        if ((rc = dpx_mc_directions((uint32_t)seed, D, dirs.data()))) return rc;
        const int rule = h->ctx->conv_rule;
        const int64_t samples = h->ctx->conv_samples;
        h->ctx->conv_rule = DPX_CONV_GPU;
        h->ctx->conv_samples = 4096;  // ITERS_PER_KERNEL of GPUHybridCalc.cu:204
        rc = dpx_orientation_average(h->ctx, nm, grids.data(), rot.data(), tr.data(), ncop.data(), crot.data(),
                                     ctr.data(), sscale.data(), nq, h->Q.data(), dirs.data(), 0, 0, D, epsi,
                                     outData);
        h->ctx->conv_rule = rule;
        h->ctx->conv_samples = samples;
    } else {
        rc = dpx_vegas_intensity(h->ctx, nm, grids.data(), rot.data(), tr.data(), ncop.data(), crot.data(),
                                 ctr.data(), sscale.data(), nq, h->Q.data(), seed, 4096, iterations, epsi, outData);
    }
    if (!rc && pStop && *pStop) rc = fail(DPX_ERR_STOPPED, "stopped");
    return rc;
}

int dpx_hybrid_destroy(dpx_hybrid h) {
    if (!h) return fail(DPX_ERR_ARG, "hybrid calculator is NULL");
    hybrid_free(h);
    return DPX_OK;
}

}  // extern "C"
