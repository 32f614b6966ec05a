// shim_driver.cpp — test infrastructure: calls D+'s GPU entry points, as the
// reference's own call sites declare them (its headers), through the libdpx
// shims of dplus-dev_gb300/shims/dplus_gpu_shims.cpp.  Prints one line per
// entry point: its return value and dpx_last_error().  Without a GPU each call
// must come back with libdpx's "no device" status mapped to the reference's
// failure value; with one, with success.
#include "GPUHeader.h"
#include "InternalGPUHeaders.h"
#include "PDBAmplitudeCUDA.h"
#include "dpx.h"

#include <cstdio>
#include <vector>

bool GPUHybrid_PDBAmplitudeDLL(GridWorkspace& work);

int main() {
    const int gs = 20, L = gs / 2, lp = L + 3;
    const long long voxels = 6LL * lp * (lp + 1) * (lp + 1) + 1;
    const double qmax = 5.0, step = qmax / L;
    // two carbon atoms (the International Tables X-ray coefficients of C)
    float coeffs[9] = {2.31f, 20.8439f, 1.02f, 10.2075f, 1.5886f, 0.5687f, 0.865f, 51.6512f, 0.2156f};
    int api[1] = {2};
    atomicFFCalculator aff(1, 2, 1, coeffs, api);
    std::vector<float4> atoms = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.15f, 0.f, 0.f, 0.f)};
    std::vector<double> grid(2 * voxels), ders(2 * voxels);
    int rc = PDBJacobianGridAmplitudeCalculation(voxels, 3, 6, (float)step, grid.data(), atoms, aff, {}, {}, 0.f,
                                                 0.05, {}, {}, 0.0, 1.0, nullptr, nullptr, 0.f, 1.f, nullptr);
    std::printf("fill %d %s\n", rc, dpx_last_error());
    std::vector<double> qs = {0.5, 1.0, 2.0}, I(3);
    rc = GPUCalcMCOAJacobSphrDD(voxels, 3, 6, step, grid.data(), ders.data(), qs.data(), I.data(), 3, 1000, 0.0,
                                nullptr, nullptr, 0.f, 1.f, nullptr);
    std::printf("mcoa %d %s\n", rc, dpx_last_error());
    IGPUGridCalculator* calc = GPUCreateCalculatorHybrid();
    std::vector<GridWorkspace> ws(1);
    std::vector<float> q = {0.5f, 1.0f, 2.0f};
    const bool ok = calc->Initialize(0, q, 2 * voxels, 3, 6, L + 4, qmax, step, ws[0]);
    std::printf("hybrid_init %d %s\n", ok ? 1 : 0, dpx_last_error());
    if (ok) {
        calc->SetNumChildren(ws[0], 1);
        GridWorkspace& child = ws[0].children[0];
        calc->Initialize(0, q, 2 * voxels, 3, 6, L + 4, qmax, step, child);
        child.atomsPerIon = api;
        child.numUniqueIons = 1;
        std::vector<float> affs((L + 4) * 1);
        aff.GetQMajorAFFMatrix(affs.data(), L + 4, (float)step);
        GPUHybrid_SetPDB(child, atoms, affs, 0.0, nullptr, nullptr, 0, 0.05f, nullptr, nullptr, 0, 0.f);
        const bool filled = GPUHybrid_PDBAmplitudeDLL(child);
        std::vector<float4> rots = {make_float4(0.f, 0.f, 0.f, 1.f)}, trans = {make_float4(0.f, 0.f, 0.f, 0.f)};
        calc->AddRotations(child, rots);
        calc->AddTranslations(child, 0, trans);
        ws[0].intMethod = OA_MC;
        const bool done = calc->ComputeIntensity(ws, I.data(), 1e-3, 100000, nullptr, nullptr, 0.f, 1.f, nullptr);
        std::printf("hybrid_run %d %d %.9g %.9g\n", filled ? 1 : 0, done ? 1 : 0, I[0], I[2]);
        calc->FreeWorkspace(ws[0]);
    }
    return 0;
}
