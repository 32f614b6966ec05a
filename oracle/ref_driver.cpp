/*
 * ref_driver.cpp — C entry points over the reference's own JacobianSphereGrid
 * and atomicFFCalculator, compiled from the unmodified reference sources
 * (Backend/Backend/Grid.cpp, Backend/GPU/Atomic Form Factor.cpp,
 * Common/mathfuncs.cpp, Backend/Backend/backend_exception.cpp) by
 * oracle/Makefile into oracle/_ref/libdplus_ref.so.
 *
 * TEST INFRASTRUCTURE ONLY: used in the build container to pin the oracle's
 * restatement against the reference itself.  Nothing here ships.
 *
 * The glue below (the per-cell amplitude callback) mirrors
 * PDBAmplitude::calcAmplitude (PDBAmplitude.cpp:243-317, atoms + dummy-atom
 * solvent branch) in the reference's own float arithmetic, because
 * PDBAmplitude.cpp itself needs Boost and does not build here.
 */
#include "Grid.h"
#include "Atomic Form Factor.h"

#include <complex>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

extern "C" {

/* Fill a reference grid with the float calcAmplitude and run its own
 * CalculateSplines (JacobianSphereGrid::Fill, Grid.cpp:760-828). */
int ref_grid_fill(int grid_size, double qmax, int n_atoms, const float* xyz, int U, const int* atoms_per_ion,
                  const float* coeffs, const float* ion_rads, int flags, float sol_ed, float c1, double scale,
                  double* out_data, double* out_coeffs) {
    JacobianSphereGrid grid((unsigned short)grid_size, qmax);
    Eigen::Matrix<float, Eigen::Dynamic, 3> atomLocs(n_atoms, 3);
    for (int j = 0; j < n_atoms; j++)
        for (int k = 0; k < 3; k++) atomLocs(j, k) = xyz[3 * j + k];
    std::vector<float> fc(coeffs, coeffs + 9 * U);
    std::vector<int> api(atoms_per_ion, atoms_per_ion + U);
    std::vector<float> rads(ion_rads, ion_rads + U);
    atomicFFCalculator aff(flags, n_atoms, U, fc.data(), api.data());
    if (flags & CALC_DUMMY_SOLVENT) aff.SetSolventED(sol_ed, c1, rads.data(), false);

    auto calc = [&](double qx, double qy, double qz) -> std::complex<double> {
        double q = std::sqrt(qx * qx + qy * qy + qz * qz), resI = 0.0, resR = 0.0;
        Eigen::Matrix<float, 3, 1> qVec(qx, qy, qz);
        Eigen::Array<float, -1, 1> phases = (atomLocs * qVec).array();
        Eigen::Array<float, Eigen::Dynamic, 1> affs(n_atoms);
        aff.GetAllAFFs(affs.data(), q);
        resI += (affs * phases.sin()).sum();
        resR += (affs * phases.cos()).sum();
        return std::complex<double>(resR, resI) * scale;
    };
    grid.Fill(calc, nullptr, nullptr, 0.0, 1.0, nullptr);
    long long n = (long long)(grid.GetRealSize() / sizeof(double));
    std::memcpy(out_data, grid.GetDataPointer(), sizeof(double) * n);
    std::memcpy(out_coeffs, grid.GetInterpolantPointer(), sizeof(double) * n);
    return 0;
}

/* The reference's CalculateSplines on given grid values (Grid.cpp:1113-1151). */
int ref_grid_splines(int grid_size, double qmax, const double* data, double* out_coeffs) {
    JacobianSphereGrid grid((unsigned short)grid_size, qmax);
    long long n = (long long)(grid.GetRealSize() / sizeof(double));
    std::memcpy(grid.GetDataPointer(), data, sizeof(double) * n);
    grid.CalculateSplines();
    std::memcpy(out_coeffs, grid.GetInterpolantPointer(), sizeof(double) * n);
    return 0;
}

/* The reference's getAmplitudesAtPoints with given values and coefficients
 * (Grid.cpp:677-721). */
int ref_grid_amplitudes_at_points(int grid_size, double qmax, const double* data, const double* coeffs, int nq,
                                  const double* qs, double theta, double phi, double* out) {
    JacobianSphereGrid grid((unsigned short)grid_size, qmax);
    long long n = (long long)(grid.GetRealSize() / sizeof(double));
    std::memcpy(grid.GetDataPointer(), data, sizeof(double) * n);
    grid.CalculateSplines();
    std::memcpy(grid.GetInterpolantPointer(), coeffs, sizeof(double) * n);
    std::vector<double> q(qs, qs + nq);
    ArrayXcX r = grid.getAmplitudesAtPoints(q, theta, phi);
    for (int k = 0; k < nq; k++) {
        out[2 * k] = r(k).real();
        out[2 * k + 1] = r(k).imag();
    }
    return 0;
}

/* GetSphr single-point interpolation (Grid.cpp:487-548). */
int ref_grid_sphr(int grid_size, double qmax, const double* data, const double* coeffs, int n,
                  const double* q_th_ph, double* out) {
    JacobianSphereGrid grid((unsigned short)grid_size, qmax);
    long long sz = (long long)(grid.GetRealSize() / sizeof(double));
    std::memcpy(grid.GetDataPointer(), data, sizeof(double) * sz);
    grid.CalculateSplines();
    std::memcpy(grid.GetInterpolantPointer(), coeffs, sizeof(double) * sz);
    for (int k = 0; k < n; k++) {
        std::complex<double> v = grid.GetSphr(q_th_ph[3 * k], q_th_ph[3 * k + 1], q_th_ph[3 * k + 2]);
        out[2 * k] = v.real();
        out[2 * k + 1] = v.imag();
    }
    return 0;
}

/* The reference's q-major unique-ion form-factor table (Atomic Form Factor.cpp:58-64). */
int ref_aff_qmajor(int U, const int* atoms_per_ion, const float* coeffs, const float* ion_rads, int flags,
                   float sol_ed, float c1, int nq, float step, float* out) {
    int n_atoms = 0;
    for (int u = 0; u < U; u++) n_atoms += atoms_per_ion[u];
    std::vector<float> fc(coeffs, coeffs + 9 * U);
    std::vector<int> api(atoms_per_ion, atoms_per_ion + U);
    std::vector<float> rads(ion_rads, ion_rads + U);
    atomicFFCalculator aff(flags, n_atoms, U, fc.data(), api.data());
    if (flags & CALC_DUMMY_SOLVENT) aff.SetSolventED(sol_ed, c1, rads.data(), false);
    std::vector<float> m(nq * U);
    aff.GetQMajorAFFMatrix(m.data(), nq, step);
    /* GetQMajorAFFMatrix maps an [nq x U] column-major array; return it q-major */
    for (int k = 0; k < nq; k++)
        for (int u = 0; u < U; u++) out[k * U + u] = m[k + u * nq];
    return 0;
}

/* The reference's binary amplitude file, version 13: JacobianSphereGrid::
 * ExportBinaryData (Grid.cpp:847-890) of the given values. */
int ref_amp_write(const char* path, const char* header, int grid_size, double qmax, const double* data) {
    JacobianSphereGrid grid((unsigned short)grid_size, qmax);
    long long n = (long long)(grid.GetRealSize() / sizeof(double));
    std::memcpy(grid.GetDataPointer(), data, sizeof(double) * n);
    std::ofstream f(path, std::ios::binary);
    return grid.ExportBinaryData(f, std::string(header ? header : "")) ? 0 : -1;
}

/* JacobianSphereGrid::ImportBinaryData (Grid.cpp:892-963) into a grid of
 * (grid_size, qmax): the values, the step it read and the header text. */
int ref_amp_read(const char* path, int grid_size, double qmax, double* out_data, double* step, char* header,
                 int header_cap) {
    JacobianSphereGrid grid((unsigned short)grid_size, qmax);
    std::ifstream f(path, std::ios::binary);
    std::string head;
    if (!grid.ImportBinaryData(f, head)) return -1;
    long long n = (long long)(grid.GetRealSize() / sizeof(double));
    std::memcpy(out_data, grid.GetDataPointer(), sizeof(double) * n);
    *step = grid.GetStepSize();
    if (header && header_cap > 0) {
        std::strncpy(header, head.c_str(), (size_t)header_cap - 1);
        header[header_cap - 1] = 0;
    }
    return 0;
}

}  // extern "C"
