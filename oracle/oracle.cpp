/*
 * oracle.cpp — CPU restatement of D+'s scattering hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load this library; libdpx never does.
 *
 * Each routine restates a reference algorithm (uri-raviv-lab/dplus-dev) and
 * cites the file:line it follows.  Self-contained C++17 + OpenMP so that it
 * builds on any host (no Eigen, no reference headers).
 */
#include "oracle.h"

#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <random>
#include <vector>
#include <algorithm>
#include <array>
#include <climits>
#include <unordered_map>
#include <omp.h>

namespace {

typedef std::complex<double> cd;
const double kPi = 3.14159265358979323846;
const double k2Pi = 6.28318530717958647692528676656;

/* ------------------------------------------------------------------------ */
/* Grid geometry.  Shell i (1..L') holds (3i+1) theta rows x 6i phi points;  */
/* the origin is cell 0 (Grid.cpp:169-200, IndexFromIndices :1078-1084).     */
/* ------------------------------------------------------------------------ */
struct Geom {
    int L;        /* radial layers = grid_size / 2 */
    int Lp;       /* layers incl. the 3 extra shells (Extras = 3, Grid.cpp:221) */
    double step;  /* qmax / L (Grid.cpp:177) */
    int64_t P;    /* number of complex cells */
};

Geom make_geom(int grid_size, double qmax) {
    Geom g;
    g.L = grid_size / 2;
    g.Lp = g.L + 3;
    g.step = qmax / double(g.L);
    int64_t lp = g.Lp;
    g.P = 6 * lp * (lp + 1) * (lp + 1) + 1;
    return g;
}

inline int64_t shell_base(int64_t i) {  /* first cell of shell i >= 1 */
    return 1 + 6 * (i - 1) * i * i;
}

/* Reference adds 8 to the bit pattern of a positive double before truncation
 * (Grid.cpp:149-150, 500-501, 559-560, 698-699). */
inline double bump8(double x) {
    int64_t b;
    std::memcpy(&b, &x, 8);
    b += 8;
    std::memcpy(&x, &b, 8);
    return x;
}

/* ------------------------------------------------------------------------ */
/* Form factors (Atomic Form Factor.cpp:121-176 internalAtomicFF, solvent    */
/* contrast :91-115 default branch, r_m :11-27).                             */
/* ------------------------------------------------------------------------ */
template <typename R>
void unique_affs(int U, const double* coeffs, const R rm, const double* ion_rads, int flags,
                 double sol_ed, double c1, R q, R* out) {
    const R sqq = (q * q / (R(100.0) * R(157.913670417429737901351855998)));
    for (int u = 0; u < U; u++) {
        R f = 0;
        if (flags & ORC_CALC_ATOMIC_FORMFACTORS) {
            R s = 0;
            for (int k = 0; k < 4; k++) {
                R a = R(coeffs[u + (2 * k) * U]);
                R b = R(coeffs[u + (2 * k + 1) * U]);
                s += std::exp(-sqq * b) * a;
            }
            f = s + R(coeffs[u + 8 * U]);
        }
        R solvent = 0;
        if (flags & ORC_CALC_DUMMY_SOLVENT) {
            R r = R(ion_rads[u]);
            R cc1 = R(c1);
            solvent = R(4.1887902047863909846) * r * r * r *
                      std::exp(-((rm * rm) * (q * q) * R(0.2067834969664667))) * R(sol_ed);
            solvent *= cc1 * cc1 * cc1 *
                       std::exp(R(-0.6822178052976590) * q * q * rm * rm * (cc1 * cc1 - R(1.0)));
        }
        out[u] = f - solvent;
    }
}

template <typename R>
R mean_radius(int U, const int* atoms_per_ion, const double* ion_rads) {
    /* r_m = cbrt(sum r^3 n / sum n) (Atomic Form Factor.cpp:23) */
    R s = 0, n = 0;
    for (int u = 0; u < U; u++) {
        R r = R(ion_rads[u]);
        s += r * r * r * R(atoms_per_ion[u]);
        n += R(atoms_per_ion[u]);
    }
    return std::cbrt(s / n);
}

/* ------------------------------------------------------------------------ */
/* calcAmplitude (PDBAmplitude.cpp:243-317), atoms + dummy-atom solvent.     */
/* ------------------------------------------------------------------------ */
struct Structure {
    int64_t N;
    const double* xyz;
    int U;
    const int* atoms_per_ion;
    const double* coeffs;
    const double* ion_rads;
    int flags;
    double sol_ed, c1, scale;
};

cd amp_fp64(const Structure& s, double rm, double qx, double qy, double qz) {
    double q = std::sqrt(qx * qx + qy * qy + qz * qz);
    double aff[64];
    unique_affs<double>(s.U, s.coeffs, rm, s.ion_rads, s.flags, s.sol_ed, s.c1, q, aff);
    double re = 0, im = 0;
    int64_t j = 0;
    for (int u = 0; u < s.U; u++) {
        double sr = 0, si = 0;
        for (int64_t e = j + s.atoms_per_ion[u]; j < e; j++) {
            double ph = qx * s.xyz[3 * j] + qy * s.xyz[3 * j + 1] + qz * s.xyz[3 * j + 2];
            sr += std::cos(ph);
            si += std::sin(ph);
        }
        re += aff[u] * sr;
        im += aff[u] * si;
    }
    return cd(re, im) * s.scale;
}

/* Reference-exact: float phases, float sin/cos and float sums, the per-atom
 * form factor evaluated in float at float(q) (PDBAmplitude.cpp:244-273). */
cd amp_refexact(const Structure& s, const float* fxyz, float rm, double qx, double qy, double qz) {
    double qd = std::sqrt(qx * qx + qy * qy + qz * qz);
    float q = float(qd);
    float aff[64];
    unique_affs<float>(s.U, s.coeffs, rm, s.ion_rads, s.flags, s.sol_ed, s.c1, q, aff);
    float fx = float(qx), fy = float(qy), fz = float(qz);
    float sr = 0, si = 0;
    int64_t j = 0;
    for (int u = 0; u < s.U; u++) {
        for (int64_t e = j + s.atoms_per_ion[u]; j < e; j++) {
            float ph = fxyz[3 * j] * fx + fxyz[3 * j + 1] * fy + fxyz[3 * j + 2] * fz;
            si += aff[u] * std::sin(ph);
            sr += aff[u] * std::cos(ph);
        }
    }
    double resI = 0.0 + si, resR = 0.0 + sr;
    return cd(resR, resI) * s.scale;
}

/* Cell -> q vector as JacobianSphereGrid::Fill computes it (Grid.cpp:797-822). */
inline void cell_qvec(const Geom& g, int qi, int64_t thi, int64_t phi, double& qx, double& qy, double& qz) {
    if (qi == 0) { qx = qy = qz = 0.0; return; }
    double qI = double(qi) * g.step;
    double tI = kPi * double(thi) / double(3 * qi);
    double pI = k2Pi * double(phi) / double(6 * qi);
    double cst = std::cos(tI), snt = std::sin(tI), csp = std::cos(pI), snp = std::sin(pI);
    qx = qI * snt * csp;
    qy = qI * snt * snp;
    qz = qI * cst;
}

void fill_range(const Geom& g, const Structure& s, int mode, int nthreads, int shell_lo, int shell_hi,
                double* data) {
    int64_t lo = (shell_lo <= 0) ? 0 : shell_base(shell_lo);
    int64_t hi = shell_base(int64_t(shell_hi) + 1);  /* exclusive */
    if (hi > g.P) hi = g.P;
    std::vector<float> fxyz;
    if (mode == ORC_REFEXACT) {
        fxyz.resize(3 * s.N);
        for (int64_t k = 0; k < 3 * s.N; k++) fxyz[k] = float(s.xyz[k]);
    }
    double rm = mean_radius<double>(s.U, s.atoms_per_ion, s.ion_rads);
    float rmf = mean_radius<float>(s.U, s.atoms_per_ion, s.ion_rads);
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ind = lo; ind < hi; ind++) {
        int qi; int64_t ti, pi;
        orc_indices_from_index(ind, &qi, &ti, &pi);
        double qx, qy, qz;
        cell_qvec(g, qi, ti, pi, qx, qy, qz);
        cd v = (mode == ORC_REFEXACT) ? amp_refexact(s, fxyz.data(), rmf, qx, qy, qz)
                                      : amp_fp64(s, rm, qx, qy, qz);
        data[2 * ind] = v.real();
        data[2 * ind + 1] = v.imag();
    }
}

/* ------------------------------------------------------------------------ */
/* Periodic cubic spline derivatives along phi (PeriodicSplineSolver.h:7-67). */
/* Solves circ(1,4,1) d = 3 (y[k+1] - y[k-1]).  FP64 mode: the same          */
/* elimination in double; reference-exact: the diagonal/right column kept    */
/* in float as the reference does.                                           */
/* ------------------------------------------------------------------------ */
template <typename DiagT>
void periodic_spline(const cd* y, cd* res, int64_t n) {
    std::vector<cd> as(n);
    std::vector<DiagT> diag(n, DiagT(4)), rc(n > 1 ? n - 1 : 1, DiagT(0));
    for (int64_t i = 0; i < n; i++) as[i] = 3.0 * (y[(i + 1) % n] - y[(n + i - 1) % n]);
    rc[0] = 1;
    rc[n - 2] = 1;
    double vp = 0.25, vc;
    for (int64_t i = 1; i < n - 1; i++) {
        vc = 1.0 / (double(diag[i]) - vp);
        diag[i] = DiagT(double(diag[i]) - vp);
        rc[i] = DiagT(double(rc[i]) - vp * double(rc[i - 1]));
        as[i] -= as[i - 1] * vp;
        vp = vc;
    }
    diag[n - 1] = DiagT(double(diag[n - 1]) - vp * double(rc[n - 2]));
    as[n - 1] -= vp * as[n - 2];
    DiagT bottom_left = 1;
    for (int64_t i = 0; i < n - 1; i++) {
        vc = double(bottom_left) / double(diag[i]);
        diag[n - 1] = DiagT(double(diag[n - 1]) - vc * double(rc[i]));
        as[n - 1] -= vc * as[i];
        bottom_left = DiagT(-vc);
    }
    double fac = double(rc[n - 2]) / double(diag[n - 1]);
    as[n - 2] -= as[n - 1] * fac;
    for (int64_t i = n - 3; i >= 0; i--) {
        as[i] -= as[n - 1] * double(DiagT(double(rc[i]) / double(diag[n - 1])));
        as[i] -= as[i + 1] * double(DiagT(1.0 / double(diag[i + 1])));
    }
    for (int64_t i = 0; i < n; i++) res[i] = as[i] / double(diag[i]);
}

/* ------------------------------------------------------------------------ */
/* Interpolation (Grid.cpp:61-134 InterpolateThetaPhiPlane, 1220-1256).      */
/* ------------------------------------------------------------------------ */
struct GridView {
    Geom g;
    const double* data;
    const double* coeffs;
    cd val(int64_t cell) const { return cd(data[2 * cell], data[2 * cell + 1]); }
    cd der(int64_t cell) const { return cd(coeffs[2 * cell], coeffs[2 * cell + 1]); }
};

inline void four_point(cd y1, cd y2, cd y3, cd y4, cd& d2, cd& d3) {
    /* PeriodicSplineSolver.h:227-234 (Ginsburg et al. 2019, eqs 35-36) */
    d2 = -(7. / 15.) * (y2 - y1) + (14. / 15.) * (y3 - y1) - (4. / 15.) * (y4 - y2) + (2. / 15.) * (y4 - y3);
    d3 = (2. / 15.) * (y2 - y1) - (4. / 15.) * (y3 - y1) + (14. / 15.) * (y4 - y2) - (7. / 15.) * (y4 - y3);
}

inline cd hermite(cd p1, cd p2, cd d1, cd d2, double t) {
    return p1 + d1 * t + (3.0 * (p2 - p1) - 2.0 * d1 - d2) * (t * t) + (2.0 * (p1 - p2) + d1 + d2) * (t * t * t);
}

cd interp_plane(const GridView& G, int ri, double theta, double phi) {
    const int64_t base = shell_base(ri);
    const int64_t phiPoints = 6 * int64_t(ri), thePoints = 3 * int64_t(ri);
    const double edge = k2Pi / double(phiPoints);
    int64_t tI = (int64_t)((theta / kPi) * double(thePoints));
    int64_t pI = (int64_t)((phi / k2Pi) * double(phiPoints));
    double tTh = (theta / edge) - double(tI);
    double tPh = (phi / edge) - double(pI);
    if (std::fabs(tTh) < 1.0e-10) tTh = 0.0;
    if (std::fabs(tPh) < 1.0e-10) tPh = 0.0;
    if (pI == phiPoints) pI = 0;
    const int64_t pI1 = (pI + 1) % phiPoints;
    cd nodes[4];
    for (int i = -1; i < 3; i++) {
        int64_t theInd = (thePoints + 1 + tI + i) % (thePoints + 1);
        int64_t c1, c2;
        if (theInd == tI + i) {
            c1 = base + phiPoints * theInd + pI;
            c2 = base + phiPoints * theInd + pI1;
        } else {
            /* wrapped row: the reference shifts by half a ring (Grid.cpp:95-105) */
            if (tI + i > thePoints) theInd = (tI + i) - (thePoints + 1);
            c1 = base + phiPoints * theInd + pI;
            c2 = base + phiPoints * theInd + pI1;
            c1 += ((2 * pI >= phiPoints) ? -phiPoints : phiPoints) / 2;
            c2 += ((2 * pI1 >= phiPoints) ? -phiPoints : phiPoints) / 2;
        }
        nodes[i + 1] = hermite(G.val(c1), G.val(c2), G.der(c1), G.der(c2), tPh);
    }
    cd ds1, ds2;
    four_point(nodes[0], nodes[1], nodes[2], nodes[3], ds1, ds2);
    return hermite(nodes[1], nodes[2], ds1, ds2, tTh);
}

/* GetSplineBetweenPlanes (Grid.cpp:551-607) */
int spline_between_planes(const GridView& G, double q, double th, double ph, cd& pl1, cd& pl2, cd& d1, cd& d2) {
    double frc = bump8(std::fabs(q) / G.g.step);
    int fInd = int(frc);
    cd plane1, plane2, plane3, plane4;
    cd origin = G.val(0);
    if (fInd == 0) {
        double new_th = kPi - th;
        double new_phi = ph + kPi;
        if (new_phi < 0) new_phi = k2Pi + (new_phi - int(new_phi / k2Pi) * k2Pi);
        if (new_phi >= k2Pi) new_phi = new_phi - int(new_phi / k2Pi) * k2Pi;
        if (new_th < 0) new_th = 0.;
        if (new_th > kPi) new_th = kPi;
        plane1 = interp_plane(G, fInd + 1, new_th, new_phi);
    } else if (fInd == 1) {
        plane1 = origin;
    } else {
        plane1 = interp_plane(G, fInd - 1, th, ph);
    }
    plane2 = (fInd > 0) ? interp_plane(G, fInd, th, ph) : origin;
    plane3 = interp_plane(G, fInd + 1, th, ph);
    plane4 = (fInd + 2 < G.g.Lp) ? interp_plane(G, fInd + 2, th, ph) : plane3;
    four_point(plane1, plane2, plane3, plane4, d1, d2);
    pl1 = plane2;
    pl2 = plane3;
    return std::max(fInd, 0);
}

/* getAmplitudesAtPoints (Grid.cpp:677-721) */
void grid_amps_at_points(const GridView& G, int nq, const double* qs, double theta, double phi, cd* out) {
    int i = 0;
    while (i < nq) {
        cd pl1, pl2, d1, d2;
        int planeIndex = spline_between_planes(G, qs[i], theta, phi, pl1, pl2, d1, d2);
        double q0 = qs[i];
        int k = i;
        while (k < nq && qs[k] < q0 + G.g.step) {
            double frc = bump8(qs[k] / G.g.step);
            double frac = frc - double(planeIndex);
            out[k] = hermite(pl1, pl2, d1, d2, frac);
            k++;
        }
        i = k;
    }
}

/* GetSphr (Grid.cpp:487-548), the single-q path used through GetCart. */
cd grid_sphr(const GridView& G, double rr, double th, double ph) {
    if (rr == 0.0) return G.val(0);
    double frc = bump8(rr / G.g.step);
    int fInd = int(frc);
    double frac = frc - double(fInd);
    cd plane2 = (fInd > 0) ? interp_plane(G, fInd, th, ph) : G.val(0);
    if (frac < 1.e-9) return plane2;
    cd pl1, pl2, d1, d2;
    spline_between_planes(G, rr, th, ph, pl1, pl2, d1, d2);
    return hermite(pl1, pl2, d1, d2, frac);
}

/* EulerD, Tait-Bryan X1Y2Z3 (Amplitude.h:557-573) */
void euler_d(double a, double b, double c, double R[9]) {
    double c1 = std::cos(a), s1 = std::sin(a), c2 = std::cos(b), s2 = std::sin(b), c3 = std::cos(c), s3 = std::sin(c);
    R[0] = c2 * c3;           R[1] = -c2 * s3;          R[2] = s2;
    R[3] = c1 * s3 + c3 * s1 * s2; R[4] = c1 * c3 - s1 * s2 * s3; R[5] = -c2 * s1;
    R[6] = s1 * s3 - c1 * c3 * s2; R[7] = c3 * s1 + c1 * s2 * s3; R[8] = c1 * c2;
}

inline void row_times(const double v[3], const double R[9], double out[3]) {
    /* out = v^T R */
    out[0] = v[0] * R[0] + v[1] * R[3] + v[2] * R[6];
    out[1] = v[0] * R[1] + v[1] * R[4] + v[2] * R[7];
    out[2] = v[0] * R[2] + v[1] * R[5] + v[2] * R[8];
}

inline void dir_to_angles(const double v[3], double& th, double& ph) {
    double z = v[2];
    if (z > 1.0) z = 1.0;
    if (z < -1.0) z = -1.0;
    th = std::acos(z);
    ph = std::atan2(v[1], v[0]);
    if (ph < 0.0) ph += kPi * 2.;
}

/* Amplitude::getAmplitudesAtPoints for a grid leaf (Amplitude.cpp:3553-3600):
 * rotate the direction by the leaf's RotMat, phase e^{i q (Qt.R)}. */
void leaf_amps(const GridView& G, const double Rm[9], const double tr[3], int nq, const double* qs,
               double theta, double phi, cd* out, std::vector<cd>& tmp) {
    double st = std::sin(theta), ct = std::cos(theta), sp = std::sin(phi), cp = std::cos(phi);
    /* the reference forms Q (st cp, st sp, ct) R / Q; the unit direction gives
     * the same vector and stays defined at q = 0 */
    double qc[3] = {st * cp, st * sp, ct}, qt[3];
    row_times(qc, Rm, qt);
    double nth, nph;
    dir_to_angles(qt, nth, nph);
    double dotR = qt[0] * tr[0] + qt[1] * tr[1] + qt[2] * tr[2];
    tmp.resize(nq);
    grid_amps_at_points(G, nq, qs, nth, nph, tmp.data());
    for (int k = 0; k < nq; k++) out[k] = tmp[k] * std::exp(cd(0., 1.) * (dotR * qs[k]));
}

struct LeafModel {
    GridView G;
    double R[9];
    double tr[3];
    int n_copies;
    std::vector<std::array<double, 9>> copyR;
    std::vector<std::array<double, 3>> copyT;
    std::vector<std::vector<int>> groups;  /* copies grouped by identical rotation */
    double sym_scale;
};

/* ManualSymmetry::getAmplitudesAtPoints (Symmetries.cpp:1079-1166): the
 * symmetry node itself sits at identity; each unique rotation is applied to
 * the direction, the translation phases use the original direction. */
void model_amps(const LeafModel& M, int nq, const double* qs, double theta, double phi, cd* out,
                std::vector<cd>& tmp, std::vector<cd>& tmp2) {
    if (M.n_copies == 0) {
        leaf_amps(M.G, M.R, M.tr, nq, qs, theta, phi, out, tmp);
        return;
    }
    double st = std::sin(theta), ct = std::cos(theta), sp = std::sin(phi), cp = std::cos(phi);
    double dir[3] = {st * cp, st * sp, ct};
    for (int k = 0; k < nq; k++) out[k] = 0;
    tmp2.resize(nq);
    for (const auto& grp : M.groups) {
        const auto& Rk = M.copyR[grp[0]];
        double qn[3];
        row_times(dir, Rk.data(), qn);
        double nrm = std::sqrt(qn[0] * qn[0] + qn[1] * qn[1] + qn[2] * qn[2]);
        qn[0] /= nrm; qn[1] /= nrm; qn[2] /= nrm;
        double nth, nph;
        dir_to_angles(qn, nth, nph);
        leaf_amps(M.G, M.R, M.tr, nq, qs, nth, nph, tmp2.data(), tmp);
        for (int k = 0; k < nq; k++) {
            cd ph(0, 0);
            for (int c : grp) {
                const auto& t = M.copyT[c];
                double a = dir[0] * t[0] + dir[1] * t[1] + dir[2] * t[2];
                ph += std::exp(cd(0., 1.) * (a * qs[k]));
            }
            out[k] += tmp2[k] * ph;
        }
    }
    for (int k = 0; k < nq; k++) out[k] *= M.sym_scale;
}

LeafModel make_model(int grid_size, double qmax, const orc_leaf& L) {
    LeafModel M;
    M.G.g = make_geom(grid_size, qmax);
    M.G.data = L.data;
    M.G.coeffs = L.coeffs;
    euler_d(L.rot[0], L.rot[1], L.rot[2], M.R);
    for (int k = 0; k < 3; k++) M.tr[k] = L.tr[k];
    M.n_copies = L.n_copies;
    M.sym_scale = L.sym_scale;
    for (int c = 0; c < L.n_copies; c++) {
        std::array<double, 9> R;
        euler_d(L.copy_rot[3 * c], L.copy_rot[3 * c + 1], L.copy_rot[3 * c + 2], R.data());
        M.copyR.push_back(R);
        M.copyT.push_back({L.copy_tr[3 * c], L.copy_tr[3 * c + 1], L.copy_tr[3 * c + 2]});
        int found = -1;
        for (size_t g = 0; g < M.groups.size(); g++) {
            int r = M.groups[g][0];
            if (L.copy_rot[3 * r] == L.copy_rot[3 * c] && L.copy_rot[3 * r + 1] == L.copy_rot[3 * c + 1] &&
                L.copy_rot[3 * r + 2] == L.copy_rot[3 * c + 2]) { found = int(g); break; }
        }
        if (found < 0) M.groups.push_back({c});
        else M.groups[found].push_back(c);
    }
    return M;
}

/* Amplitude::getAmplitude through GetCart (Amplitude.cpp:3035-3056,
 * Grid.cpp:384-392), used by the GK integrand. */
cd leaf_amp_cart(const LeafModel& M, double qx, double qy, double qz) {
    auto one = [&](const double dirq[3]) -> cd {
        double qt[3];
        row_times(dirq, M.R, qt);
        double r = std::sqrt(qt[0] * qt[0] + qt[1] * qt[1] + qt[2] * qt[2]);
        if (std::fabs(qt[2]) > r) r = std::fabs(qt[2]);
        double th = (r == 0.0) ? 0.0 : std::acos(qt[2] / r);
        double ph = std::atan2(qt[1], qt[0]);
        if (ph < 0.0) ph += k2Pi;
        double a = dirq[0] * M.tr[0] + dirq[1] * M.tr[1] + dirq[2] * M.tr[2];
        return std::exp(cd(0., 1.) * a) * grid_sphr(M.G, r, th, ph);
    };
    double Q[3] = {qx, qy, qz};
    if (M.n_copies == 0) return one(Q);
    /* ManualSymmetry::calcAmplitude (Symmetries.cpp:697-716) */
    cd res(0, 0);
    for (int c = 0; c < M.n_copies; c++) {
        double qn[3];
        row_times(Q, M.copyR[c].data(), qn);
        cd ri = one(qn);
        const auto& t = M.copyT[c];
        res += ri * std::exp(cd(0., 1.) * (Q[0] * t[0] + Q[1] * t[1] + Q[2] * t[2]));
    }
    return res * M.sym_scale;
}

/* Gauss-Kronrod (7,15) abscissae and weights (the standard published rule,
 * as used by DomainModel::GaussLegTheta/Phi). */
const double kX15[15] = {
    -0.9914553711208126392068547, -0.9491079123427585245261897, -0.8648644233597690727897128,
    -0.7415311855993944398638648, -0.5860872354676911302941448, -0.4058451513773971669066064,
    -0.2077849550078984676006894, 0.0, 0.2077849550078984676006894, 0.4058451513773971669066064,
    0.5860872354676911302941448, 0.7415311855993944398638648, 0.8648644233597690727897128,
    0.9491079123427585245261897, 0.9914553711208126392068547};
const double kW15[15] = {
    0.0229353220105292249637320, 0.0630920926299785532907007, 0.1047900103222501838398763,
    0.1406532597155259187451896, 0.1690047266392679028265834, 0.1903505780647854099132564,
    0.2044329400752988924141620, 0.2094821410847278280129992, 0.2044329400752988924141620,
    0.1903505780647854099132564, 0.1690047266392679028265834, 0.1406532597155259187451896,
    0.1047900103222501838398763, 0.0630920926299785532907007, 0.0229353220105292249637320};
const double kW7[7] = {
    0.1294849661688696932706114, 0.2797053914892766679014678, 0.3818300505051189449503698,
    0.4179591836734693877551020, 0.3818300505051189449503698, 0.2797053914892766679014678,
    0.1294849661688696932706114};

struct GKCtx {
    std::vector<LeafModel>* models;
};

double gk_phi(const GKCtx& C, double q, double st, double ct, double pMin, double pMax, double eps,
              int64_t maxDepth, int64_t minDepth) {
    /* DomainModel::GaussLegPhi (Amplitude.cpp:1445-1467) */
    cd kv[15];
    double kVal = 0.0, gVal = 0.0, ba = pMax - pMin, apb = pMax + pMin, ba2 = ba * 0.5, apb2 = apb * 0.5;
    for (int i = 0; i < 15; i++) {
        double xi = apb2 + ba2 * kX15[i];
        kv[i] = 0;
        for (auto& M : *C.models) kv[i] += leaf_amp_cart(M, q * st * std::cos(xi), q * st * std::sin(xi), q * ct);
        kVal += std::real(kv[i] * std::conj(kv[i])) * ba2 * kW15[i];
        if (i % 2 == 1) gVal += std::real(kv[i] * std::conj(kv[i])) * ba2 * kW7[i / 2];
    }
    if (minDepth < 0 && (maxDepth < 0 || std::fabs(1.0 - (gVal / kVal)) <= eps || gVal == kVal)) return kVal;
    return gk_phi(C, q, st, ct, pMin, apb2, eps, maxDepth - 1, minDepth - 1) +
           gk_phi(C, q, st, ct, apb2, pMax, eps, maxDepth - 1, minDepth - 1);
}

double gk_theta(const GKCtx& C, double q, double tMin, double tMax, double eps, int64_t maxDepth, int64_t minDepth) {
    /* DomainModel::GaussLegTheta (Amplitude.cpp:1421-1443) */
    double kVal = 0.0, gVal = 0.0, ba = tMax - tMin, apb = tMax + tMin, ba2 = ba * 0.5, apb2 = apb * 0.5;
    for (int i = 0; i < 15; i++) {
        double sT = std::sin(apb2 + ba2 * kX15[i]);
        double v = gk_phi(C, q, sT, std::cos(apb2 + ba2 * kX15[i]), 0.0, k2Pi, eps, maxDepth, minDepth);
        kVal += v * kW15[i] * ba2 * sT;
        if (i % 2 == 1) gVal += v * kW7[i / 2] * ba2 * sT;
    }
    if (minDepth < 0 && (maxDepth < 0 || std::fabs(1.0 - (gVal / kVal)) <= eps || gVal == kVal)) return kVal;
    double mid = (tMax + tMin) / 2.0;
    return gk_theta(C, q, tMin, mid, eps, maxDepth - 1, minDepth - 1) +
           gk_theta(C, q, mid, tMax, eps, maxDepth - 1, minDepth - 1);
}

}  // namespace

/* ======================================================================== */
extern "C" {

int64_t orc_grid_cells(int grid_size) { return make_geom(grid_size, 1.0).P; }

int64_t orc_index_from_indices(int qi, int64_t ti, int64_t pi) {
    if (qi == 0) return 0;
    return shell_base(qi) + ti * 6 * int64_t(qi) + pi;
}

void orc_indices_from_index(int64_t index, int* qi, int64_t* ti, int64_t* pi) {
    /* inverse of shell_base: largest i with 1 + 6(i-1)i^2 <= index */
    if (index == 0) { *qi = 0; *ti = 0; *pi = 0; return; }
    int64_t i = (int64_t)std::cbrt(double(index) / 6.0);
    if (i < 1) i = 1;
    while (i > 1 && shell_base(i) > index) i--;
    while (shell_base(i + 1) <= index) i++;
    int64_t rem = index - shell_base(i);
    *qi = int(i);
    *ti = rem / (6 * i);
    *pi = rem % (6 * i);
}

void orc_aff_table(int U, const double* coeffs, const int* atoms_per_ion, const double* ion_rads, int flags,
                   double sol_ed, double c1, int nq, double q0, double dq, int mode, double* out) {
    if (mode == ORC_REFEXACT) {
        float rm = mean_radius<float>(U, atoms_per_ion, ion_rads);
        std::vector<float> tmp(U);
        for (int k = 0; k < nq; k++) {
            /* GetQMajorAFFMatrix evaluates at float(qMin + stepSize*i) (Atomic Form Factor.cpp:58-64) */
            float q = float(q0) + float(dq) * float(k);
            unique_affs<float>(U, coeffs, rm, ion_rads, flags, sol_ed, c1, q, tmp.data());
            for (int u = 0; u < U; u++) out[k * U + u] = tmp[u];
        }
    } else {
        double rm = mean_radius<double>(U, atoms_per_ion, ion_rads);
        for (int k = 0; k < nq; k++)
            unique_affs<double>(U, coeffs, rm, ion_rads, flags, sol_ed, c1, q0 + dq * k, out + k * U);
    }
}

void orc_grid_fill_shells(int grid_size, double qmax, int64_t N, const double* xyz, int U,
                          const int* atoms_per_ion, const double* coeffs, const double* ion_rads, int flags,
                          double sol_ed, double c1, double scale, int mode, int nthreads, int shell_lo,
                          int shell_hi, double* data) {
    Geom g = make_geom(grid_size, qmax);
    Structure s{N, xyz, U, atoms_per_ion, coeffs, ion_rads, flags, sol_ed, c1, scale};
    fill_range(g, s, mode, nthreads, shell_lo, shell_hi, data);
}

void orc_grid_fill(int grid_size, double qmax, int64_t N, const double* xyz, int U, const int* atoms_per_ion,
                   const double* coeffs, const double* ion_rads, int flags, double sol_ed, double c1,
                   double scale, int mode, int nthreads, double* data) {
    Geom g = make_geom(grid_size, qmax);
    orc_grid_fill_shells(grid_size, qmax, N, xyz, U, atoms_per_ion, coeffs, ion_rads, flags, sol_ed, c1,
                         scale, mode, nthreads, 0, g.Lp, data);
}

/* Voxelized-solvent boxes added to every cell (PDBAmplitude.cpp:277-314):
 *   data += scale * sum_b w_b prod_a [L_a sinc(q_a L_a / 2)] e^{i q.c_b}
 * boxes: 8 floats per box {cx, cy, cz, w, Lx, Ly, Lz, 0}.  FP64 mode promotes
 * the box floats to double; reference-exact mode evaluates in float as the
 * reference's Eigen float arrays do (sinc = sin(x)/x, 1 where that is NaN). */
void orc_grid_add_boxes_shells(int grid_size, double qmax, int64_t n_boxes, const float* boxes, double scale,
                               int mode, int nthreads, int shell_lo, int shell_hi, double* data) {
    Geom g = make_geom(grid_size, qmax);
    int64_t lo = (shell_lo <= 0) ? 0 : shell_base(shell_lo);
    int64_t hi = shell_base(int64_t(shell_hi) + 1); /* exclusive */
    if (hi > g.P) hi = g.P;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ind = lo; ind < hi; ind++) {
        int qi; int64_t ti, pi;
        orc_indices_from_index(ind, &qi, &ti, &pi);
        double qx, qy, qz;
        cell_qvec(g, qi, ti, pi, qx, qy, qz);
        double re = 0, im = 0;
        if (mode == ORC_REFEXACT) {
            const float q[3] = {float(qx), float(qy), float(qz)};
            float fr = 0.f, fi = 0.f;
            for (int64_t b = 0; b < n_boxes; b++) {
                const float* B = boxes + 8 * b;
                float va = 1.f, ph = 0.f;
                for (int a = 0; a < 3; a++) {
                    const float x = B[4 + a] * (0.5f * q[a]);
                    float sc = std::sin(x) / x;
                    if (sc != sc) sc = 1.f;
                    va *= sc * B[4 + a];
                    ph += B[a] * q[a];
                }
                va *= B[3];
                fr += va * std::cos(ph);
                fi += va * std::sin(ph);
            }
            re = fr;
            im = fi;
        } else {
            const double q[3] = {qx, qy, qz};
            for (int64_t b = 0; b < n_boxes; b++) {
                const float* B = boxes + 8 * b;
                double va = B[3], ph = 0;
                for (int a = 0; a < 3; a++) {
                    const double L = B[4 + a], x = 0.5 * q[a] * L;
                    va *= L * (x == 0.0 ? 1.0 : std::sin(x) / x);
                    ph += q[a] * double(B[a]);
                }
                re += va * std::cos(ph);
                im += va * std::sin(ph);
            }
        }
        data[2 * ind] += scale * re;
        data[2 * ind + 1] += scale * im;
    }
}

void orc_grid_add_boxes(int grid_size, double qmax, int64_t n_boxes, const float* boxes, double scale, int mode,
                        int nthreads, double* data) {
    Geom g = make_geom(grid_size, qmax);
    orc_grid_add_boxes_shells(grid_size, qmax, n_boxes, boxes, scale, mode, nthreads, 0, g.Lp, data);
}

void orc_grid_splines(int grid_size, const double* data, double* coeffs, int mode, int nthreads) {
    Geom g = make_geom(grid_size, 1.0);
    coeffs[0] = coeffs[1] = 0.0;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 1; i <= g.Lp; i++) {
        int64_t rows = 3 * int64_t(i) + 1;
        for (int64_t j = 0; j < rows; j++) {
            int64_t pos = orc_index_from_indices(i, j, 0);
            const cd* y = reinterpret_cast<const cd*>(data + 2 * pos);
            cd* r = reinterpret_cast<cd*>(coeffs + 2 * pos);
            if (mode == ORC_REFEXACT) periodic_spline<float>(y, r, 6 * int64_t(i));
            else periodic_spline<double>(y, r, 6 * int64_t(i));
        }
    }
}

void orc_grid_amplitudes_at_points(int grid_size, double qmax, const double* data, const double* coeffs, int nq,
                                   const double* qs, double theta, double phi, double* out) {
    GridView G{make_geom(grid_size, qmax), data, coeffs};
    grid_amps_at_points(G, nq, qs, theta, phi, reinterpret_cast<cd*>(out));
}

void orc_mc_directions(uint32_t seed, int64_t D, double* theta_phi) {
    std::mt19937 rng;
    rng.seed(seed);
    std::uniform_real_distribution<double> ranU2(0.0, 2.0);
    for (int64_t i = 0; i < D; i++) {
        double u2 = ranU2(rng);
        double v2 = ranU2(rng);
        theta_phi[2 * i + 1] = u2 * kPi;
        theta_phi[2 * i] = std::acos(v2 - 1.0);
    }
}

void orc_layer_seeds(uint32_t master, int nq, int n_layers, uint32_t* seeds) {
    std::mt19937 seedGen;
    std::uniform_int_distribution<unsigned int> sRan(0, UINT_MAX);
    seedGen.seed(master);
    for (int i = 0; i < nq; i++) (void)sRan(seedGen);
    for (int i = 0; i < n_layers + 1; i++) seeds[i] = sRan(seedGen);
}

void orc_q_brackets(int grid_size, double qmax, int nq, const double* Q, int* layer_of_q) {
    const int L = grid_size / 2;
    const double stepSize = 2 * qmax / grid_size;
    for (int k = 0; k < nq; k++) layer_of_q[k] = -1;
    int tmpLayer = 0;
    while (Q[0] > (tmpLayer + 1) * stepSize) tmpLayer++;
    for (int layer = tmpLayer; layer < L; layer++) {
        int qb = 0;
        while (qb < nq && Q[qb] <= layer * stepSize) qb++;
        if (qb >= nq) continue;
        int qe = qb + 1;
        if (qe == nq) qe--;
        while (qe + 1 != nq && Q[qe] <= (layer + 1) * stepSize) qe++;
        if (qe + 1 != nq) qe--;
        for (int k = qb; k <= qe; k++) layer_of_q[k] = layer;
    }
}

namespace {
int integrate_layers_impl(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, int nq, const double* Q,
                          const double* dirs, int64_t dir_layer_stride, int64_t max_iter, double eps, int nthreads,
                          int64_t gpu_step, double* res);
}  // namespace

int orc_integrate_layers(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, int nq, const double* Q,
                         const double* dirs, int64_t dir_layer_stride, int64_t max_iter, double eps, int nthreads,
                         double* res) {
    return integrate_layers_impl(grid_size, qmax, n_leaves, leaves, nq, Q, dirs, dir_layer_stride, max_iter, eps,
                                 nthreads, 0, res);
}

int orc_integrate_layers_gpu_rule(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, int nq,
                                  const double* Q, const double* dirs, int64_t dir_layer_stride, int64_t max_iter,
                                  double eps, int64_t samples_per_step, int nthreads, double* res) {
    if (samples_per_step <= 0) return -1;
    return integrate_layers_impl(grid_size, qmax, n_leaves, leaves, nq, Q, dirs, dir_layer_stride, max_iter, eps,
                                 nthreads, samples_per_step, res);
}

namespace {
int integrate_layers_impl(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, int nq, const double* Q,
                          const double* dirs, int64_t dir_layer_stride, int64_t max_iter, double eps, int nthreads,
                          int64_t gpu_step, double* res) {
    std::vector<LeafModel> models;
    for (int l = 0; l < n_leaves; l++) models.push_back(make_model(grid_size, qmax, leaves[l]));
    const int L = grid_size / 2;
    std::vector<int> layer_of_q(nq);
    orc_q_brackets(grid_size, qmax, nq, Q, layer_of_q.data());
    for (int k = 0; k < nq; k++) res[k] = 0.0;
    if (Q[0] == 0.0) {
        /* |sum of leaves at q = 0|^2 (Amplitude.cpp:1176-1182) */
        cd a(0, 0);
        std::vector<cd> t1, t2;
        double zero = 0.0;
        for (auto& M : models) {
            cd o;
            if (M.n_copies == 0) o = M.G.val(0);
            else {
                cd s(0, 0);
                for (size_t g = 0; g < M.groups.size(); g++) s += M.G.val(0) * double(M.groups[g].size());
                o = s * M.sym_scale;
            }
            (void)zero;
            a += o;
        }
        res[0] = std::real(a * std::conj(a));
    }
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int layer = 0; layer < L; layer++) {
        std::vector<int> idx;
        for (int k = 0; k < nq; k++)
            if (layer_of_q[k] == layer) idx.push_back(k);
        if (idx.empty()) continue;
        const int m = int(idx.size());
        std::vector<double> qs(m);
        for (int k = 0; k < m; k++) qs[k] = Q[idx[k]];
        const double* ld = dirs + 2 * int64_t(layer) * dir_layer_stride;
        std::vector<double> run(m, 0.0), hist(4 * m, 0.0);
        std::vector<cd> sums(m), one(m), t1, t2;
        bool done = false;
        for (int64_t i = 0; i < max_iter && !done; i++) {
            double theta = ld[2 * i], phi = ld[2 * i + 1];
            for (int k = 0; k < m; k++) sums[k] = 0;
            for (auto& M : models) {
                model_amps(M, m, qs.data(), theta, phi, one.data(), t1, t2);
                for (int k = 0; k < m; k++) sums[k] += one[k];
            }
            for (int k = 0; k < m; k++) run[k] += std::real(sums[k] * std::conj(sums[k]));
            if (eps > 0.0 && gpu_step > 0) {
                /* the reference GPU averages' test (OAJacob.cu:320-337, GPUHybridCalc.cu:705-720):
                 * the running mean after every gpu_step samples; from the 4th step on, converged
                 * when every q is within eps of its mean at each of the 3 steps before */
                if ((i + 1) % gpu_step != 0) continue;
                const int64_t step = (i + 1) / gpu_step - 1;
                const int pos = int(step % 4);
                for (int k = 0; k < m; k++) hist[pos * m + k] = run[k] / double(i + 1);
                if (step > 2) {
                    bool conv = true;
                    for (int j = 1; conv && j <= 3; j++) {
                        const int pj = int((step - j) % 4);
                        for (int k = 0; k < m; k++)
                            if (!(std::fabs(1.0 - hist[pos * m + k] / hist[pj * m + k]) <= eps)) { conv = false; break; }
                    }
                    if (conv) {
                        for (int k = 0; k < m; k++) res[idx[k]] = hist[pos * m + k];
                        done = true;
                    }
                }
                continue;
            }
            if (eps > 0.0 && i % 100 == 0) {
                int pos = int((i / 100) % 4);
                for (int k = 0; k < m; k++) hist[pos * m + k] = run[k] / double(i + 1);
                if (i >= 400) {
                    bool conv = true;
                    for (int j = 0; conv && j < 4; j++)
                        for (int k = 0; k < m; k++)
                            if (!(std::fabs(1.0 - hist[j * m + k] / hist[k]) < eps)) { conv = false; break; }
                    if (conv) {
                        for (int k = 0; k < m; k++) res[idx[k]] = hist[pos * m + k];
                        done = true;
                    }
                }
            }
        }
        if (!done)
            for (int k = 0; k < m; k++) res[idx[k]] = run[k] / double(max_iter);
    }
    return 0;
}
}  // namespace

namespace {
/* The voxelized-solvent boxes' amplitude at q in FP64 (PDBAmplitude.cpp:277-314,
 * the FP64 branch of orc_grid_add_boxes_shells), times scale. */
cd boxes_fp64(int64_t n_boxes, const float* boxes, double scale, double qx, double qy, double qz) {
    const double q[3] = {qx, qy, qz};
    double re = 0, im = 0;
    for (int64_t b = 0; b < n_boxes; b++) {
        const float* B = boxes + 8 * b;
        double va = B[3], ph = 0;
        for (int a = 0; a < 3; a++) {
            const double L = B[4 + a], x = 0.5 * q[a] * L;
            va *= L * (x == 0.0 ? 1.0 : std::sin(x) / x);
            ph += q[a] * double(B[a]);
        }
        re += va * std::cos(ph);
        im += va * std::sin(ph);
    }
    return cd(re, im) * scale;
}
}  // namespace

void orc_direct_intensity(int64_t N, const double* xyz, int U, const int* atoms_per_ion, const double* coeffs,
                          const double* ion_rads, int flags, double sol_ed, double c1, double scale, int64_t n_boxes,
                          const float* boxes, int n_copies, const double* copy_rot, const double* copy_tr, int nq,
                          const double* Q, int64_t D, const double* dirs, int nthreads, double* res) {
    Structure s{N, xyz, U, atoms_per_ion, coeffs, ion_rads, flags, sol_ed, c1, scale};
    auto leaf_amp = [&](double rm_, double qx, double qy, double qz) {
        cd f = amp_fp64(s, rm_, qx, qy, qz);
        if (n_boxes > 0) f += boxes_fp64(n_boxes, boxes, scale, qx, qy, qz);
        return f;
    };
    double rm = mean_radius<double>(U, atoms_per_ion, ion_rads);
    std::vector<std::array<double, 9>> Rk;
    for (int c = 0; c < n_copies; c++) {
        std::array<double, 9> R;
        euler_d(copy_rot[3 * c], copy_rot[3 * c + 1], copy_rot[3 * c + 2], R.data());
        Rk.push_back(R);
    }
    if (nthreads > 0) omp_set_num_threads(nthreads);
    for (int k = 0; k < nq; k++) {
        double acc = 0.0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
        for (int64_t d = 0; d < D; d++) {
            double th = dirs[2 * d], ph = dirs[2 * d + 1];
            double n[3] = {std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th)};
            double q = Q[k];
            cd F(0, 0);
            if (n_copies == 0) {
                F = leaf_amp(rm, q * n[0], q * n[1], q * n[2]);
            } else {
                for (int c = 0; c < n_copies; c++) {
                    double nn[3];
                    row_times(n, Rk[c].data(), nn);
                    cd f = leaf_amp(rm, q * nn[0], q * nn[1], q * nn[2]);
                    double a = q * (n[0] * copy_tr[3 * c] + n[1] * copy_tr[3 * c + 1] + n[2] * copy_tr[3 * c + 2]);
                    F += f * std::exp(cd(0., 1.) * a);
                }
            }
            acc += std::real(F * std::conj(F));
        }
        res[k] = acc / double(D);
    }
}

double orc_uniform(uint64_t seed, uint64_t key, uint64_t n) {
    /* SplitMix64 finalizer (Steele, Lea & Flood 2014) over a keyed counter */
    auto mix = [](uint64_t x) {
        x += 0x9E3779B97F4A7C15ull;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        return x ^ (x >> 31);
    };
    const uint64_t s = mix(seed ^ (key * 0xD1342543DE82EF95ull));
    return double(mix(s + n) >> 11) * (1.0 / 9007199254740992.0);
}

namespace {
/* ResizeVegasPoints (HybridOA.cu:182-268) for one dimension of n bins */
void vegas_resize(double* bounds, const double* var, int n) {
    double total = 0;
    for (int i = 0; i < n; i++) total += var[i];
    if (total == 0.) return;
    std::vector<double> w(n), nb(n, bounds[n]);
    for (int i = 0; i < n; i++) {
        double b;
        if (i == 0) b = (var[0] + var[1]) / 2.;
        else if (i == n - 1) b = (var[n - 1] + var[n - 2]) / 2.;
        else b = (var[i - 1] + var[i] + var[i + 1]) / 3.;
        double r = total / b;
        w[i] = std::pow((r - 1.) / (r * std::log(r)), 1.5);
        if (w[i] != w[i]) w[i] = 0.;
    }
    double tw = 0;
    for (int i = 0; i < n; i++) tw += w[i];
    double xold, xnew = 0., dw = 0., pts = tw / n;
    int j = 0;
    for (int i = 0; i < n; i++) {
        dw += w[i];
        xold = xnew;
        xnew = bounds[i + 1];
        for (; dw > pts; j++) {
            dw -= pts;
            if (j < n) nb[j] = xnew - dw * (xnew - xold) / w[i];
        }
    }
    for (int k = 0; k < n - 1; k++) bounds[1 + k] = nb[k];
}
}  // namespace

int orc_vegas_intensity(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, int nq, const double* Q,
                        uint64_t seed, int points_per_iter, int64_t max_points, double eps, double* res) {
    const int TB = 32, PB = 32, NB = TB * PB;
    if (points_per_iter <= 0 || points_per_iter % NB) return -1;
    const int ppb = points_per_iter / NB;
    std::vector<LeafModel> models;
    for (int l = 0; l < n_leaves; l++) models.push_back(make_model(grid_size, qmax, leaves[l]));
    const double step = qmax / (grid_size / 2);
    std::vector<double> bounds(TB + PB + 2);
    for (int i = 0; i <= TB; i++) bounds[i] = double(i) / TB;
    for (int i = 0; i <= PB; i++) bounds[1 + TB + i] = double(i) / PB;
    double* tb = bounds.data();
    double* pb = bounds.data() + TB + 1;
    int qInd = 0, lower = 0, bracket = 0;
    std::vector<cd> t1, t2, one, amp;
    do {
        /* GPUHybridCalc.cu:365-375 */
        while (Q[qInd] > double(lower + 1) * step) lower++;
        int qEnd;
        for (qEnd = qInd + 1; qEnd < nq; qEnd++)
            if (Q[qEnd] > double(lower + 1) * step) break;
        qEnd--;
        const int m = qEnd - qInd + 1;
        const double* qs = Q + qInd;
        std::vector<double> I((size_t)points_per_iter * m), run(m, 0.0);
        std::vector<std::vector<double>> hist;
        one.resize(m);
        amp.resize(m);
        for (int it = 0;; it++) {
            const uint64_t key = (uint64_t(bracket) << 32) | uint64_t(it);
            for (int p = 0; p < points_per_iter; p++) {
                const int bin = p / ppb, th = bin / PB, ph = bin % PB;
                const double r1 = orc_uniform(seed, key, 2 * uint64_t(p)), r2 = orc_uniform(seed, key, 2 * uint64_t(p) + 1);
                const double theta = std::acos(1. - 2. * (r1 * (tb[th + 1] - tb[th]) + tb[th]));
                const double phi = (r2 * (pb[ph + 1] - pb[ph]) + pb[ph]) * 2. * kPi;
                for (int k = 0; k < m; k++) amp[k] = 0;
                for (auto& M : models) {
                    model_amps(M, m, qs, theta, phi, one.data(), t1, t2);
                    for (int k = 0; k < m; k++) amp[k] += one[k];
                }
                for (int k = 0; k < m; k++) I[(size_t)p * m + k] = std::real(amp[k] * std::conj(amp[k]));
            }
            /* HybridVEGASBinReduceToIKernel / HybridVEGASBinReduceKernel (HybridOA.cu:301-449) */
            std::vector<double> est(m, 0.0), thv(TB, 0.0), phv(PB, 0.0);
            for (int bin = 0; bin < NB; bin++) {
                const int th = bin / PB, ph = bin % PB;
                const double vol = (tb[th + 1] - tb[th]) * (pb[ph + 1] - pb[ph]);
                for (int k = 0; k < m; k++) {
                    double s = 0;
                    for (int p = 0; p < ppb; p++) s += I[(size_t)(bin * ppb + p) * m + k];
                    est[k] += s * (vol / ppb);
                }
                double mean = 0, m2 = 0;
                for (int p = 0; p < ppb; p++) {
                    double sq = 0;
                    for (int k = 0; k < m; k++) sq += I[(size_t)(bin * ppb + p) * m + k];
                    const double diff = vol * sq - mean;
                    mean += diff / double(p + 1);
                    m2 += diff * diff * double(p) / double(p + 1);
                }
                thv[th] += m2 * ppb;
                phv[ph] += m2 * ppb;
            }
            vegas_resize(tb, thv.data(), TB);
            if (PB > 2) vegas_resize(pb, phv.data(), PB);
            for (int k = 0; k < m; k++) run[k] = (it == 0) ? est[k] : (run[k] * it + est[k]) / (it + 1);
            hist.push_back(run);
            bool conv = false;
            if (it > 2 && eps > 0.0) { /* checkConvergenceOA (GPUHybridCalc.cu:706-720) */
                conv = true;
                for (int k = 0; k < m && conv; k++)
                    for (int d = 1; d <= 3; d++)
                        if (std::fabs(1.0 - run[k] / hist[it - d][k]) > eps) { conv = false; break; }
            }
            if (conv || int64_t(it + 1) * points_per_iter >= max_points) break;
        }
        for (int k = 0; k < m; k++) res[qInd + k] = run[k];
        qInd = qEnd + 1;
        lower++;
        bracket++;
    } while (qInd < nq);
    return 0;
}

void orc_assemble_grid(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, const double* lattice,
                       double scale, int nthreads, double* out) {
    std::vector<LeafModel> models;
    for (int l = 0; l < n_leaves; l++) models.push_back(make_model(grid_size, qmax, leaves[l]));
    Geom g = make_geom(grid_size, qmax);
    const cd One(1.0, 0.0), Im(0.0, 1.0);
    if (nthreads > 0) omp_set_num_threads(nthreads);
    /* Grid::Fill over ManualSymmetry / Amplitude::getAmplitude (Symmetries.cpp:697-716,
     * Amplitude.cpp:3035-3056) and GridSymmetry::calcAmplitude (Symmetries.cpp:105-137) */
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ind = 0; ind < g.P; ind++) {
        int qi; int64_t ti, pi;
        orc_indices_from_index(ind, &qi, &ti, &pi);
        double qx, qy, qz;
        cell_qvec(g, qi, ti, pi, qx, qy, qz);
        cd amp(0, 0);
        for (auto& M : models) amp += leaf_amp_cart(M, qx, qy, qz);
        if (lattice) {
            for (int a = 0; a < 3; a++) {
                const double* v = lattice + 3 * a;
                const double N = lattice[9 + a];
                const double dot = qx * v[0] + qy * v[1] + qz * v[2];
                if (std::fabs(dot) < 100.0 * 2.220446049250313e-16 || N == 1.0) amp *= N;
                else amp *= (One - std::exp(Im * dot * N)) / (One - std::exp(Im * dot));
            }
        }
        amp *= scale;
        out[2 * ind] += amp.real();
        out[2 * ind + 1] += amp.imag();
    }
}

/* Debye sum, DebyeCalTester::Calculate (PDBAmplitude.cpp:1789-1825) and its
 * anomalous twin (PDBAmplitude.cpp:2466-2512): per-atom form factors at q
 * (GetAllAFFs, Atomic Form Factor.cpp), plus f' + i f'' when given, times the
 * Debye-Waller factor exp(-B (q/10)^2 / (16 pi^2)) when B factors are given;
 * I = sum_i |f_i|^2 + 2 sum_{i<j} Re(f_i conj f_j) sinc(q r_ij).  FP64: every
 * step in double.  REFEXACT: float form factors, float coordinates and
 * distances, float sinc with sin(x)/x = NaN -> 1 (SincArrayXf, Amplitude.h:108),
 * float pair products cast to double and summed in double, the self terms
 * summed in float, as the reference's Eigen expressions do. */
void orc_debye(int64_t N, const double* xyz, int U, const int* atoms_per_ion, const double* coeffs,
               const double* ion_rads, int flags, double sol_ed, double c1, const double* bfactor,
               const double* anom, int nq, const double* Q, int mode, int nthreads, double* out) {
    std::vector<int> ion(N);
    {
        int64_t j = 0;
        for (int u = 0; u < U; u++)
            for (int k = 0; k < atoms_per_ion[u]; k++) ion[j++] = u;
    }
    if (nthreads > 0) omp_set_num_threads(nthreads);
    const double rm = mean_radius<double>(U, atoms_per_ion, ion_rads);
    const float rmf = mean_radius<float>(U, atoms_per_ion, ion_rads);
    for (int k = 0; k < nq; k++) {
        const double q = Q[k];
        if (mode == ORC_REFEXACT) {
            std::vector<float> aff(U), fr(N), fi(N, 0.f);
            unique_affs<float>(U, coeffs, rmf, ion_rads, flags, sol_ed, c1, (float)q, aff.data());
            for (int64_t i = 0; i < N; i++) {
                fr[i] = aff[ion[i]];
                if (anom) {
                    fr[i] += (float)anom[2 * i];
                    fi[i] = (float)anom[2 * i + 1];
                }
                if (bfactor) {
                    const double q10 = q / 10.0;
                    const double dw = std::exp(-(bfactor[i] * q10 * q10 / (16. * kPi * kPi)));
                    fr[i] = (float)(fr[i] * dw);
                    fi[i] = (float)(fi[i] * dw);
                }
            }
            double res = 0.0;
#pragma omp parallel for reduction(+ : res) schedule(dynamic, 64)
            for (int64_t i = 1; i < N; i++) {
                const float xi = (float)xyz[3 * i], yi = (float)xyz[3 * i + 1], zi = (float)xyz[3 * i + 2];
                double row = 0.0;
                for (int64_t j = 0; j < i; j++) {
                    const float dx = (float)xyz[3 * j] - xi, dy = (float)xyz[3 * j + 1] - yi,
                                dz = (float)xyz[3 * j + 2] - zi;
                    const float x = (float)q * std::sqrt(dx * dx + dy * dy + dz * dz);
                    float sc = std::sin(x) / x;
                    if (sc != sc) sc = 1.f;
                    row += (double)(fr[i] * fr[j] + fi[i] * fi[j]) * (double)sc;
                }
                res += 2.0 * row;
            }
            float self = 0.f;
            for (int64_t i = 0; i < N; i++) self += fr[i] * fr[i] + fi[i] * fi[i];
            out[k] = res + (double)self;
        } else {
            std::vector<double> aff(U), fr(N), fi(N, 0.0);
            unique_affs<double>(U, coeffs, rm, ion_rads, flags, sol_ed, c1, q, aff.data());
            for (int64_t i = 0; i < N; i++) {
                fr[i] = aff[ion[i]];
                if (anom) {
                    fr[i] += anom[2 * i];
                    fi[i] = anom[2 * i + 1];
                }
                if (bfactor) {
                    const double q10 = q / 10.0;
                    const double dw = std::exp(-(bfactor[i] * q10 * q10 / (16. * kPi * kPi)));
                    fr[i] *= dw;
                    fi[i] *= dw;
                }
            }
            double res = 0.0;
#pragma omp parallel for reduction(+ : res) schedule(dynamic, 64)
            for (int64_t i = 1; i < N; i++) {
                double row = 0.0;
                for (int64_t j = 0; j < i; j++) {
                    const double dx = xyz[3 * j] - xyz[3 * i], dy = xyz[3 * j + 1] - xyz[3 * i + 1],
                                 dz = xyz[3 * j + 2] - xyz[3 * i + 2];
                    const double x = q * std::sqrt(dx * dx + dy * dy + dz * dz);
                    const double sc = x == 0.0 ? 1.0 : std::sin(x) / x;
                    row += (fr[i] * fr[j] + fi[i] * fi[j]) * sc;
                }
                res += 2.0 * row;
            }
            double self = 0.0;
            for (int64_t i = 0; i < N; i++) self += fr[i] * fr[i] + fi[i] * fi[i];
            out[k] = res + self;
        }
    }
}

double orc_gk_intensity(int grid_size, double qmax, int n_leaves, const orc_leaf* leaves, double q, double eps,
                        int64_t max_depth) {
    std::vector<LeafModel> models;
    for (int l = 0; l < n_leaves; l++) models.push_back(make_model(grid_size, qmax, leaves[l]));
    if (q == 0.0) {
        cd a(0, 0);
        for (auto& M : models) a += leaf_amp_cart(M, 0, 0, 0);
        return std::real(a * std::conj(a));
    }
    GKCtx C{&models};
    /* GaussKron2DSphereRecurs (Amplitude.cpp:1416-1419): theta in [0, pi/2], / 2pi */
    return gk_theta(C, q, 0.0, kPi / 2, eps, max_depth - 1, -1) / (2.0 * kPi);
}

/* Synthetic workload structures: the seeded globule every configuration is
 * built from (a self-avoiding random walk of 0.15 nm steps folded into a
 * sphere, no two atoms closer than 0.1 nm, elements C 63 / N 17 / O 19 / S 1 %),
 * the same generator the library's dpx_make_globule runs, so that the CPU
 * baseline builds its inputs without loading the library. */
int orc_make_globule(int64_t n_atoms, double radius_nm, uint64_t seed, float* xyz, int* elem) {
    if (n_atoms <= 0 || !(radius_nm > 0) || !xyz || !elem) return -1;
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U01(0.0, 1.0);
    const double step = 0.15, min_d = 0.1, cell = 0.2, R = radius_nm;
    const int64_t nc = (int64_t)std::ceil(2 * R / cell) + 2;
    auto cell_of = [&](double v) { return (int64_t)std::floor((v + R) / cell) + 1; };
    std::unordered_map<int64_t, std::vector<int64_t>> cells;
    cells.reserve((size_t)n_atoms * 2);
    auto free_at = [&](double x, double y, double z) {
        const int64_t ix = cell_of(x), iy = cell_of(y), iz = cell_of(z);
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    auto it = cells.find(((ix + dx) * nc + (iy + dy)) * nc + (iz + dz));
                    if (it == cells.end()) continue;
                    for (int64_t j : it->second) {
                        const double ex = xyz[3 * j] - x, ey = xyz[3 * j + 1] - y, ez = xyz[3 * j + 2] - z;
                        if (ex * ex + ey * ey + ez * ez < min_d * min_d) return false;
                    }
                }
        return true;
    };
    double px = 0, py = 0, pz = 0;
    for (int64_t i = 0; i < n_atoms; ++i) {
        double x = px, y = py, z = pz;
        if (i > 0) {
            bool placed = false;
            for (int attempt = 0; attempt < 64 && !placed; ++attempt) {
                const double ct = 2 * U01(rng) - 1, ph = 2 * kPi * U01(rng), st = std::sqrt(1 - ct * ct);
                x = px + step * st * std::cos(ph);
                y = py + step * st * std::sin(ph);
                z = pz + step * ct;
                if (x * x + y * y + z * z > R * R) continue;
                placed = free_at(x, y, z);
            }
            if (!placed) {  /* a dead end restarts the walk at a random free point */
                for (int attempt = 0; attempt < 100000; ++attempt) {
                    x = (2 * U01(rng) - 1) * R;
                    y = (2 * U01(rng) - 1) * R;
                    z = (2 * U01(rng) - 1) * R;
                    if (x * x + y * y + z * z <= R * R && free_at(x, y, z)) {
                        placed = true;
                        break;
                    }
                }
                if (!placed) return -1;
            }
        }
        xyz[3 * i] = (float)x;
        xyz[3 * i + 1] = (float)y;
        xyz[3 * i + 2] = (float)z;
        cells[(cell_of(x) * nc + cell_of(y)) * nc + cell_of(z)].push_back(i);
        px = x;
        py = y;
        pz = z;
        const double r = U01(rng);
        elem[i] = r < 0.63 ? 0 : (r < 0.80 ? 1 : (r < 0.99 ? 2 : 3));
    }
    return 0;
}

}  // extern "C"
