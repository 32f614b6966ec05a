// dpx_debye_host.cpp — C-ABI of the Debye sum (dpx_debye.cu): the
// device-resident call on a context, and the drop-in for the reference's
// GPUCalcDebyeV2 (DebyeCalculator.cu:164-372, declared in
// Backend/GPU/InternalGPUHeaders.h:60-61).
#include "dpx_host.h"

#include <cmath>
#include <cstring>
#include <vector>

using namespace dpxh;

namespace {

size_t put(std::vector<char>& h, const void* src, size_t n) {
    const size_t at = al16(h.size());
    h.resize(at + n);
    if (n && src) std::memcpy(h.data() + at, src, n);
    return at;
}

}  // namespace

extern "C" {

int dpx_debye_intensity(dpx_ctx ctx, const dpx_pdb_desc* d, const float* bfactors, const float* anomalous, int nq,
                        const double* Q, int precision, double* I) {
    if (!ctx || !d || (nq > 0 && (!Q || !I))) return fail(DPX_ERR_ARG, "NULL argument");
    if (nq < 0) return fail(DPX_ERR_ARG, "nq < 0");
    if (precision != DPX_FP32 && precision != DPX_FP64) return fail(DPX_ERR_ARG, "bad precision %d", precision);
    if (int rc = check_pdb(*d)) return rc;
    if (d->aff) return fail(DPX_ERR_ARG, "the Debye sum needs the form-factor coefficients, not a table");
    if (d->n_boxes > 0) return fail(DPX_ERR_ARG, "the Debye sum takes no voxelized-solvent boxes");
    for (int k = 0; k < nq; ++k)
        if (!(Q[k] >= 0.0) || !std::isfinite(Q[k])) return fail(DPX_ERR_ARG, "q[%d] is negative or not finite", k);
    if (nq == 0) return DPX_OK;
    if (int rc = set_device(ctx)) return rc;
    const int64_t n = d->n_atoms;
    const int64_t npad = dpx::debye_padded_atoms(n);
    const int blocks = dpx::debye_pair_blocks(npad);
    const bool fp64 = precision == DPX_FP64;
    const bool anom = anomalous != nullptr;
    // host staging: positions, ion indices, B factors, anomalous factors, form factors, q
    std::vector<char>& h = ctx->host_stage;
    h.clear();
    const size_t oPos = put(h, nullptr, (size_t)npad * sizeof(float4));
    if (!d->atoms_on_device) {
        float4* p = reinterpret_cast<float4*>(h.data() + oPos);
        for (int64_t i = 0; i < n; ++i) p[i] = make_float4(d->atoms[4 * i], d->atoms[4 * i + 1], d->atoms[4 * i + 2], 0.f);
    }
    std::vector<int> ion(n);
    for (int u = 0, j = 0; u < d->n_ions; ++u)
        for (int k = 0; k < d->atoms_per_ion[u]; ++k) ion[j++] = u;
    const size_t oIon = put(h, ion.data(), ion.size() * sizeof(int));
    const size_t oBf = bfactors ? put(h, bfactors, (size_t)n * sizeof(float)) : SIZE_MAX;
    const size_t oAn = anom ? put(h, anomalous, (size_t)n * 2 * sizeof(float)) : SIZE_MAX;
    std::vector<double> ff;
    aff_at(d->n_ions, d->atoms_per_ion, d->coeffs, d->ion_rads, d->flags, d->solvent_ed, d->c1, nq, Q, ff);
    const size_t oFf = put(h, ff.data(), ff.size() * sizeof(double));
    const size_t oQ = put(h, Q, (size_t)nq * sizeof(double));
    const size_t staged = al16(h.size());
    const size_t tbytes = (size_t)nq * npad * (fp64 ? sizeof(double) : sizeof(float));
    const size_t oFr = staged, oFi = al16(oFr + tbytes);
    const size_t oPart = al16(oFi + (anom ? tbytes : 0));
    const size_t oOut = al16(oPart + (size_t)blocks * nq * sizeof(double));
    const size_t total = oOut + (size_t)nq * sizeof(double);
    if (cudaError_t e = ctx->debye.reserve(total)) {
        cudaGetLastError();
        return fail(DPX_ERR_OOM, "Debye tables need %zu bytes (%s)", total, cudaGetErrorString(e));
    }
    char* base = static_cast<char*>(ctx->debye.p);
    cudaStream_t s = ctx->stream;
    DPX_CUDA(cudaMemcpyAsync(base, h.data(), staged, cudaMemcpyHostToDevice, s));
    if (d->atoms_on_device)  // (x, y, z, w) already float4 on the device
        DPX_CUDA(cudaMemcpyAsync(base + oPos, d->atoms, (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    dpx::DebyeArgs a{};
    a.pos = reinterpret_cast<const float4*>(base + oPos);
    a.ion = reinterpret_cast<const int*>(base + oIon);
    a.bfactor = bfactors ? reinterpret_cast<const float*>(base + oBf) : nullptr;
    a.anom = anom ? reinterpret_cast<const float2*>(base + oAn) : nullptr;
    a.ff = reinterpret_cast<const double*>(base + oFf);
    a.q = reinterpret_cast<const double*>(base + oQ);
    a.Fr = base + oFr;
    a.Fi = anom ? base + oFi : nullptr;
    a.partial = reinterpret_cast<double*>(base + oPart);
    a.out = reinterpret_cast<double*>(base + oOut);
    a.n = n;
    a.npad = npad;
    a.nq = nq;
    a.scale2 = d->scale * d->scale;
    DPX_CUDA(dpx::launch_debye(s, fp64, anom, a));
    DPX_CUDA(cudaMemcpyAsync(I, a.out, (size_t)nq * sizeof(double), cudaMemcpyDeviceToHost, s));
    DPX_CUDA(cudaStreamSynchronize(s));
    return DPX_OK;
}

int dpx_calc_debye_v2(int numQValues, float qMin, float qMax, double* outData, int numAtoms, const int* atomsPerIon,
                      const float* loc, const unsigned char* ionInd, const float* anomalousVals, int bBfactors,
                      const float* BFactors, const float* coeffs, int bSol, int bSolOnly, const char* atmInd,
                      const float* atmRad, float solvED, float c1, int precision, int* pStop) {
    (void)ionInd;  // the reference reads the ions from atomsPerIon; ionInd is unused there as well
    if (!outData || !atomsPerIon || !loc || !coeffs) return fail(DPX_ERR_ARG, "NULL buffer");
    if (numQValues <= 0 || numAtoms <= 0) return fail(DPX_ERR_ARG, "numQValues and numAtoms must be positive");
    if (bBfactors && !BFactors) return fail(DPX_ERR_ARG, "bBfactors without BFactors");
    // unique ions: atomsPerIon up to the atom count (DebyeCalculator.cu:183-185)
    int U = 0;
    int64_t tot = 0;
    while (tot < numAtoms && atomsPerIon[U] > 0) tot += atomsPerIon[U++];
    if (tot != numAtoms) return fail(DPX_ERR_ARG, "atomsPerIon does not add up to numAtoms");
    int flags = bSolOnly ? 0 : DPX_CALC_ATOMIC_FORMFACTORS;
    if (bSol && solvED != 0.0f) flags |= DPX_CALC_DUMMY_SOLVENT;
    std::vector<double> cd(9 * (size_t)U), rd(U, 0.0);
    for (int k = 0; k < 9 * U; ++k) cd[k] = coeffs[k];
    if (flags & DPX_CALC_DUMMY_SOLVENT) {  // ionRads[u] = atmRad[atmInd[first atom of u]] (:203-208)
        if (!atmInd || !atmRad) return fail(DPX_ERR_ARG, "dummy-atom solvent needs atmInd and atmRad");
        for (int u = 0, off = 0; u < U; off += atomsPerIon[u++]) rd[u] = atmRad[(int)atmInd[off]];
    }
    // q_k = qMin + k (qMax - qMin) / (numQValues - 1), in float as the reference (:188, :296)
    const float step = numQValues > 1 ? (qMax - qMin) / float(numQValues - 1) : 0.f;
    std::vector<double> q(numQValues);
    for (int k = 0; k < numQValues; ++k) q[k] = (double)(qMin + step * (float)k);
    if (pStop && *pStop) return fail(DPX_ERR_STOPPED, "stopped");
    int dev = 0;
    cudaGetDevice(&dev);
    dpx_ctx ctx;
    if (int rc = dpx_ctx_create(dev, &ctx)) return rc;
    dpx_pdb_desc d{};
    d.n_atoms = numAtoms;
    d.atoms = loc;
    d.n_ions = U;
    d.atoms_per_ion = atomsPerIon;
    d.coeffs = cd.data();
    d.ion_rads = rd.data();
    d.flags = flags;
    d.solvent_ed = solvED;
    d.c1 = c1;
    d.scale = 1.0;
    int rc = dpx_debye_intensity(ctx, &d, bBfactors ? BFactors : nullptr, anomalousVals, numQValues, q.data(),
                                 precision, outData);
    if (!rc && pStop && *pStop) rc = fail(DPX_ERR_STOPPED, "stopped");
    dpx_ctx_destroy(ctx);
    return rc;
}

}  // extern "C"
