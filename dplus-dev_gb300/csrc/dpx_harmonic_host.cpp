// dpx_harmonic_host.cpp — planning and staging of the harmonic FP32 fill
// (dpx_harmonic.cu) of one leaf: the point sets (atoms about the centre with
// their ion index; solvent boxes expanded into their voxels), the expansion
// order per shell, the chunking of the points under a scratch budget, and the
// launches.
#include "dpx_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace dpxh {

namespace {

size_t put(std::vector<char>& h, const void* src, size_t n) {
    const size_t at = al16(h.size());
    h.resize(at + n);
    if (n && src) std::memcpy(h.data() + at, src, n);
    return at;
}

// Expansion order of shell i: l_i = ceil(x + 3 x^(1/3) + 6), x = q_i R.
int order_of(double x) { return (int)std::ceil(x + 3.0 * std::cbrt(x) + 6.0); }

// Radial bin width x q_max: the degree-5 interpolation of j_l(q r) over a bin
// then errs by less than 2e-8.
constexpr double kBinWidthTimesQmax = 0.7;
// Points per moments block.
constexpr int kUnitPoints = 1024;

// Chebyshev nodes cos((2c+1) pi / 12) and the inverse of their Vandermonde
// matrix V[c][n] = x_c^n (Gauss-Jordan in double).
void chebyshev_fit(double nodes[6], double vinv[36]) {
    double a[6][12];
    for (int c = 0; c < 6; ++c) {
        nodes[c] = std::cos((2 * c + 1) * 3.14159265358979323846 / 12.0);
        double x = 1.0;
        for (int n = 0; n < 6; ++n) {
            a[c][n] = x;
            a[c][6 + n] = c == n ? 1.0 : 0.0;
            x *= nodes[c];
        }
    }
    for (int col = 0; col < 6; ++col) {
        int piv = col;
        for (int r = col + 1; r < 6; ++r)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        for (int q = 0; q < 12; ++q) std::swap(a[col][q], a[piv][q]);
        const double inv = 1.0 / a[col][col];
        for (int q = 0; q < 12; ++q) a[col][q] *= inv;
        for (int r = 0; r < 6; ++r)
            if (r != col) {
                const double f = a[r][col];
                for (int q = 0; q < 12; ++q) a[r][q] -= f * a[col][q];
            }
    }
    // T = V^-1 J: T_n = sum_c vinv[n][c] J_c
    for (int n = 0; n < 6; ++n)
        for (int c = 0; c < 6; ++c) vinv[n * 6 + c] = a[n][6 + c];
}

// The voxels of the leaf's solvent boxes (centred and counted on the device by
// harmonic_accepts), expanded and sorted by radius bin (bin width delta) on
// the device, in box order within a bin (dpx::launch_voxel_bins).  The bin
// totals come back into pinned memory; bin_voxels_finish waits for them and
// builds the units of <= kUnitPoints voxels per bin.
int bin_voxels_launch(dpx_ctx ctx, const HarmLeaf& hl, double s, double delta, int nbins, const float4** out) {
    const int64_t nb = hl.nb, nv = hl.nv;
    if (nv > INT32_MAX) return fail(DPX_ERR_ARG, "harmonic fill: %lld voxels", (long long)nv);
    const int nblk = (int)((nv + 255) / 256);
    const size_t oTmp = 0;
    const size_t oBin = al16(oTmp + (size_t)nv * sizeof(float4));
    const size_t oHist = al16(oBin + (size_t)nv * sizeof(int));
    const size_t oOff = al16(oHist + (size_t)nbins * nblk * sizeof(int));
    const size_t oTot = al16(oOff + (size_t)nbins * nblk * sizeof(int64_t));
    const size_t oOut = al16(oTot + (size_t)nbins * sizeof(int64_t));
    const size_t total = oOut + (size_t)nv * sizeof(float4);
    if (cudaError_t e = ctx->voxels.reserve(total)) {
        cudaGetLastError();
        return fail(DPX_ERR_OOM, "voxel binning needs %zu bytes (%s)", total, cudaGetErrorString(e));
    }
    char* base = static_cast<char*>(ctx->voxels.p);
    cudaStream_t st = ctx->stream;
    dpx::VoxelBinArgs a{};
    a.boxes = hl.boxes;
    a.counts = hl.counts;
    a.vstart = hl.vstart;
    a.run_sums = hl.run_sums;
    a.nb = nb;
    a.nv = nv;
    a.vs = (float)s;
    a.delta = (float)delta;
    a.nbins = nbins;
    a.tmp = reinterpret_cast<float4*>(base + oTmp);
    a.vbin = reinterpret_cast<int*>(base + oBin);
    a.hist = reinterpret_cast<int*>(base + oHist);
    a.off = reinterpret_cast<int64_t*>(base + oOff);
    a.total = reinterpret_cast<int64_t*>(base + oTot);
    a.out = reinterpret_cast<float4*>(base + oOut);
    DPX_CUDA(dpx::launch_voxel_bins(st, a));
    char* hp = nullptr;
    DPX_CUDA(ctx->pin_totals.get((size_t)nbins * sizeof(int64_t), &hp));
    DPX_CUDA(cudaMemcpyAsync(hp, a.total, (size_t)nbins * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    DPX_CUDA(ctx->pin_totals.copied(st));
    *out = a.out;
    return DPX_OK;
}

int bin_voxels_finish(dpx_ctx ctx, int nbins, std::vector<int4>& units, std::vector<int2>& groups,
                      std::vector<int>& gu) {
    char* hp = nullptr;
    DPX_CUDA(ctx->pin_totals.get((size_t)nbins * sizeof(int64_t), &hp));  // waits for the copy
    const int64_t* tot = reinterpret_cast<const int64_t*>(hp);
    int64_t start = 0;
    for (int bin = 0; bin < nbins; ++bin) {
        const int64_t c = tot[bin];
        if (c > 0) {
            gu.push_back((int)units.size());
            groups.push_back(make_int2(bin, -1));
            for (int64_t o = 0; o < c; o += kUnitPoints)
                units.push_back(make_int4((int)(start + o), (int)std::min<int64_t>(kUnitPoints, c - o), bin, 0));
        }
        start += c;
    }
    gu.push_back((int)units.size());
    return DPX_OK;
}

}  // namespace

bool harmonic_accepts(dpx_ctx ctx, int slot, const dpx_pdb_desc& d, const dpx::Geom& G,
                      std::vector<float>& host_atoms, HarmLeaf& hl, int* status) {
    *status = DPX_OK;
    hl = HarmLeaf{};
    if (d.n_boxes > 0 && d.boxes && !(d.voxel_step > 0.0)) return false;
    const float* src = d.atoms;
    if (d.atoms_on_device) {  // atoms already shifted by the centre
        host_atoms.resize((size_t)4 * d.n_atoms);
        cudaError_t e = cudaMemcpyAsync(host_atoms.data(), d.atoms, host_atoms.size() * sizeof(float),
                                        cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            *status = cuda_fail(e, "harmonic fill: atoms to host");
            return false;
        }
        src = host_atoms.data();
    }
    // the centre of stage_leaf: the given one, else the host atoms' centroid
    double c[3] = {0, 0, 0};
    if (d.center) {
        for (int k = 0; k < 3; ++k) c[k] = d.center[k];
    } else if (!d.atoms_on_device) {
        for (int64_t a = 0; a < d.n_atoms; ++a)
            for (int k = 0; k < 3; ++k) c[k] += src[4 * a + k];
        for (int k = 0; k < 3; ++k) c[k] /= (double)d.n_atoms;
    }
    const double ca[3] = {d.atoms_on_device ? 0.0 : c[0], d.atoms_on_device ? 0.0 : c[1],
                          d.atoms_on_device ? 0.0 : c[2]};
    double r2 = 0.0;
    for (int64_t a = 0; a < d.n_atoms; ++a) {
        double q = 0;
        for (int k = 0; k < 3; ++k) q += (src[4 * a + k] - ca[k]) * (src[4 * a + k] - ca[k]);
        r2 = std::max(r2, q);
    }
    double r2_pts = r2;  // the points themselves: atoms and voxel centres
    // the solvent boxes: uploaded once, centred and counted on the device, with
    // their largest corner distance and the voxel total read back
    const int64_t nb = d.n_boxes > 0 && d.boxes ? d.n_boxes : 0;
    if (nb > 0) {
        if ((int)ctx->leaf_boxes.size() <= slot) ctx->leaf_boxes.resize(slot + 1);
        dpxh::DevBuf& B = ctx->leaf_boxes[slot];
        const size_t oRaw = 0;
        const size_t oBox = al16((size_t)8 * nb * sizeof(float));
        const size_t oCnt = al16(oBox + (size_t)2 * nb * sizeof(float4));
        const size_t oVs = al16(oCnt + (size_t)nb * sizeof(int64_t));
        const size_t oRs = al16(oVs + (size_t)nb * sizeof(int64_t));
        const size_t oSc = al16(oRs + (size_t)((nb + dpx::kVoxelScanRun - 1) / dpx::kVoxelScanRun) * sizeof(int64_t));
        cudaError_t e = B.reserve(oSc + 3 * sizeof(unsigned long long));
        char* base = static_cast<char*>(B.p);
        cudaStream_t st = ctx->stream;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(base + oRaw, d.boxes, (size_t)8 * nb * sizeof(float), cudaMemcpyHostToDevice, st);
        dpx::VoxelPrepArgs a{};
        a.raw = reinterpret_cast<const float*>(base + oRaw);
        a.nb = nb;
        a.cx = c[0];
        a.cy = c[1];
        a.cz = c[2];
        a.vs = (float)d.voxel_step;
        a.boxes = reinterpret_cast<float4*>(base + oBox);
        a.counts = reinterpret_cast<int64_t*>(base + oCnt);
        a.scal = reinterpret_cast<unsigned long long*>(base + oSc);
        if (e == cudaSuccess) e = dpx::launch_voxel_prepare(st, a);
        char* hp = nullptr;
        if (e == cudaSuccess) e = ctx->pin_small.get(3 * sizeof(unsigned long long), &hp);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hp, a.scal, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            *status = cuda_fail(e, "harmonic fill: solvent boxes");
            return false;
        }
        const unsigned long long* sc = reinterpret_cast<const unsigned long long*>(hp);
        const unsigned qbits = (unsigned)sc[0], vbits = (unsigned)sc[2];
        float qf, vf;
        std::memcpy(&qf, &qbits, sizeof qf);
        std::memcpy(&vf, &vbits, sizeof vf);
        r2_pts = std::max(r2_pts, (double)vf);
        r2 = std::max(r2, (double)qf);
        hl.nb = nb;
        hl.nv = (int64_t)sc[1];
        hl.boxes = a.boxes;
        hl.counts = a.counts;
        hl.vstart = reinterpret_cast<int64_t*>(base + oVs);
        hl.run_sums = reinterpret_cast<int64_t*>(base + oRs);
    }
    // the fill's points are rounded to FP32 about the centre: a relative margin
    const double R = std::sqrt(r2) * (1.0 + 1e-6);
    hl.R = R;
    hl.R_pts = std::min(R, std::sqrt(r2_pts) * (1.0 + 1e-6));
    if (order_of(G.Lp * G.step * R) > dpx::harmonic_max_l()) return false;
    const double delta = kBinWidthTimesQmax / (G.Lp * G.step);
    if (nb > 0 && (int)(R / delta) + 1 > dpx::harmonic_max_bins()) return false;
    return true;
}

int harmonic_fill(dpx_ctx ctx, const dpx_pdb_desc& d, const LeafTables& t, const char* dbase, const dpx::Geom& G,
                  void* grid, const std::vector<float>& host_atoms, const HarmLeaf& hl) {
    const double R = hl.R;
    const int Lp = G.Lp;
    cudaStream_t st = ctx->stream;
    cudaEvent_t* ev = nullptr;  // [0, 1] atoms' moments, [2, 3] voxels' moments, [4, 5] synthesis, [6, 7] fill
    if (ctx->timing) {
        for (cudaEvent_t& e : ctx->tev)
            if (!e) DPX_CUDA(cudaEventCreate(&e));
        ev = ctx->tev;
        DPX_CUDA(cudaEventRecord(ev[6], st));
    }
    // ---- radial bins; the voxels are expanded and binned on the device while
    // the host plans the rest ----
    const double delta = kBinWidthTimesQmax / (Lp * G.step);
    const int nbins = (int)(R / delta) + 1;
    const double s = d.voxel_step;
    const float4* vox_dev = nullptr;
    if (hl.nb > 0) {
        if (nbins > dpx::harmonic_max_bins())
            return fail(DPX_ERR_ARG, "harmonic fill: %d radial bins above %d", nbins, dpx::harmonic_max_bins());
        if (int rc = bin_voxels_launch(ctx, hl, s, delta, nbins, &vox_dev)) return rc;
    }
    // ---- point sets about the leaf's centre t.cen (device atoms arrive shifted) ----
    const float* src = d.atoms_on_device ? host_atoms.data() : d.atoms;
    const double sh[3] = {d.atoms_on_device ? 0.0 : t.cen[0], d.atoms_on_device ? 0.0 : t.cen[1],
                          d.atoms_on_device ? 0.0 : t.cen[2]};
    auto centred_atoms = [&]() {
        std::vector<float4> atoms(d.n_atoms);
        int64_t j = 0;
        for (int u = 0; u < d.n_ions; ++u)
            for (int k = 0; k < d.atoms_per_ion[u]; ++k, ++j)
                atoms[j] = make_float4((float)((double)src[4 * j] - sh[0]), (float)((double)src[4 * j + 1] - sh[1]),
                                       (float)((double)src[4 * j + 2] - sh[2]), (float)u);
        return atoms;
    };
    // ---- the degree-5 interpolation of the radial bins on Chebyshev nodes ----
    double nodes[6], vinv[36];
    chebyshev_fit(nodes, vinv);
    // ---- groups: (bin, ion) for atoms, bin for voxels; counting sort ----
    struct Set {
        std::vector<float4> pts;
        std::vector<int4> units;
        std::vector<int2> groups;
        std::vector<int> gu;
    };
    auto make_set = [&](const std::vector<float4>& in, bool voxels, Set& out) {
        const int nion = voxels ? 1 : d.n_ions;
        const int ng = nbins * nion;
        std::vector<int> gid(in.size()), count(ng + 1, 0);
        for (size_t j = 0; j < in.size(); ++j) {
            const float4& p = in[j];
            const double r = std::sqrt((double)p.x * p.x + (double)p.y * p.y + (double)p.z * p.z);
            const int b = std::min(nbins - 1, (int)(r / delta));
            gid[j] = b * nion + (voxels ? 0 : (int)p.w);
            count[gid[j] + 1]++;
        }
        for (int g = 0; g < ng; ++g) count[g + 1] += count[g];
        out.pts.resize(in.size());
        std::vector<int> fill(count.begin(), count.end() - 1);
        for (size_t j = 0; j < in.size(); ++j) {
            float4 p = in[j];
            if (!voxels) p.w = 1.f;  // the ion's form factor is applied per shell
            out.pts[fill[gid[j]]++] = p;
        }
        for (int g = 0; g < ng; ++g) {
            const int n = count[g + 1] - count[g];
            if (n == 0) continue;
            out.gu.push_back((int)out.units.size());
            out.groups.push_back(make_int2(g / nion, voxels ? -1 : g % nion));
            for (int o = 0; o < n; o += kUnitPoints)
                out.units.push_back(make_int4(count[g] + o, std::min(kUnitPoints, n - o), g / nion, 0));
        }
        out.gu.push_back((int)out.units.size());
    };
    Set sa, sv;  // built after the tables and the voxels' moments are launched
    const int64_t n_vox = hl.nb > 0 ? hl.nv : 0;
    // ---- orders.  hl.R_pts bounds the atoms and the voxel centres (R, the box
    // corners, bounds the bins).  Bin b needs the orders l <= order_of(q_max
    // (b + 1) delta) only. ----
    const double Reff = hl.R_pts;
    std::vector<int> lmax(Lp + 1, 0);
    for (int i = 1; i <= Lp; ++i) lmax[i] = order_of(i * G.step * Reff);
    const int LM = lmax[Lp];
    if (LM > dpx::harmonic_max_l()) return fail(DPX_ERR_ARG, "harmonic fill: order %d above %d", LM,
                                                dpx::harmonic_max_l());
    const int K = (LM + 1) * (LM + 2) / 2;
    std::vector<int> lmb(nbins);
    for (int b = 0; b < nbins; ++b) lmb[b] = std::min(LM, order_of(Lp * G.step * (b + 1) * delta * (1.0 + 1e-6)));
    std::vector<float2> ab(K, make_float2(0.f, 0.f));
    for (int m = 0; m <= LM; ++m)
        for (int l = m + 1; l <= LM; ++l) {
            const double a = std::sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            const double b = std::sqrt((((double)l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
            ab[(size_t)l * (l + 1) / 2 + m] = make_float2((float)a, (float)b);
        }
    // the moments' scaled recurrence q_l = Pbar_lm / r_lm, r_lm = prod_{j=m+1..l} a_jm / 2:
    // q_l = 2x q_{l-1} - c_lm q_{l-2}, c_lm = 4 b_lm / a_{l-1,m} (0 for l = m + 1)
    std::vector<float2> cr(K, make_float2(0.f, 1.f));
    for (int m = 0; m <= LM; ++m) {
        double r = 1.0, a_prev = 0.0;
        for (int l = m + 1; l <= LM; ++l) {
            const double a = std::sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            const double b = std::sqrt((((double)l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
            r *= 0.5 * a;
            const double c = l >= m + 2 ? 4.0 * b / a_prev : 0.0;
            cr[(size_t)l * (l + 1) / 2 + m] = make_float2((float)c, (float)r);
            a_prev = a;
        }
    }
    std::vector<float> nmm(LM + 1);  // Pbar_mm = nmm[m] (-sin theta)^m, orthonormal
    {
        double v = 0.28209479177387814347;  // 1 / sqrt(4 pi)
        for (int m = 0; m <= LM; ++m) {
            if (m > 0) v *= std::sqrt((2.0 * m + 1.0) / (2.0 * m));
            nmm[m] = (float)v;
        }
    }
    const size_t cell_set = (size_t)(Lp + 1) * K * sizeof(float2);
    const size_t moments_per_unit = (size_t)6 * K * sizeof(float2);
    // ---- device arena ----
    std::vector<char> h;
    const size_t oL = put(h, lmax.data(), lmax.size() * sizeof(int));
    const size_t oLb = put(h, lmb.data(), lmb.size() * sizeof(int));
    const size_t oAb = put(h, ab.data(), ab.size() * sizeof(float2));
    const size_t oCr = put(h, cr.data(), cr.size() * sizeof(float2));
    const size_t oNm = put(h, nmm.data(), nmm.size() * sizeof(float));
    const size_t oNo = put(h, nodes, sizeof nodes);
    const size_t oVi = put(h, vinv, sizeof vinv);
    size_t oP[2], oU[2], oG[2], oGu[2];
    Set* sets[2] = {&sa, &sv};
    const size_t staged = al16(h.size());
    // the voxels' units, groups and group starts come with their bin totals,
    // the atoms' set once the voxels' moments run: regions sized for at most
    // one partial unit per group
    const size_t vox_units_max = n_vox ? (size_t)(n_vox + kUnitPoints - 1) / kUnitPoints + nbins : 0;
    oU[1] = staged;
    oG[1] = al16(oU[1] + vox_units_max * sizeof(int4));
    oGu[1] = al16(oG[1] + (size_t)nbins * sizeof(int2));
    oP[1] = 0;
    const size_t atom_groups_max = (size_t)nbins * d.n_ions;
    const size_t atom_units_max = (size_t)(d.n_atoms + kUnitPoints - 1) / kUnitPoints + atom_groups_max;
    oP[0] = al16(oGu[1] + (size_t)(nbins + 1) * sizeof(int));
    oU[0] = al16(oP[0] + (size_t)d.n_atoms * sizeof(float4));
    oG[0] = al16(oU[0] + atom_units_max * sizeof(int4));
    oGu[0] = al16(oG[0] + atom_groups_max * sizeof(int2));
    const size_t oJn = al16(oGu[0] + (atom_groups_max + 1) * sizeof(int));
    const size_t oT = al16(oJn + (size_t)(Lp + 1) * nbins * 6 * (LM + 1) * sizeof(double));
    const size_t oMP = al16(oT + (size_t)(Lp + 1) * nbins * (LM + 1) * 8 * sizeof(float));
    // moments scratch: the voxels' at oMP / oM, the atoms' (on the side
    // stream, at the same time) at oMPa / oMa
    const size_t oM = al16(oMP + vox_units_max * moments_per_unit);
    const size_t oMPa = al16(oM + (n_vox ? (size_t)nbins : (size_t)0) * moments_per_unit);
    const size_t oMa = al16(oMPa + atom_units_max * moments_per_unit);
    const size_t oCa = al16(oMa + atom_groups_max * moments_per_unit);
    const size_t oCv = al16(oCa + cell_set);
    const size_t total = oCv + (n_vox == 0 ? 0 : cell_set);
    if (cudaError_t e = ctx->harmonic.reserve(total)) {
        cudaGetLastError();
        return fail(DPX_ERR_OOM, "harmonic fill needs %zu bytes (%s)", total, cudaGetErrorString(e));
    }
    char* base = static_cast<char*>(ctx->harmonic.p);
    char* hp = nullptr;
    DPX_CUDA(ctx->pin_plan.get(staged, &hp));
    std::memcpy(hp, h.data(), staged);
    DPX_CUDA(cudaMemcpyAsync(base, hp, staged, cudaMemcpyHostToDevice, st));
    DPX_CUDA(ctx->pin_plan.copied(st));
    const int* d_lmax = reinterpret_cast<const int*>(base + oL);
    dpx::HarmonicTables tb{};
    tb.Lp = Lp;
    tb.nbins = nbins;
    tb.LM = LM;
    tb.step = G.step;
    tb.delta = delta;
    tb.lmax = d_lmax;
    tb.nodes = reinterpret_cast<const double*>(base + oNo);
    tb.vinv = reinterpret_cast<const double*>(base + oVi);
    tb.Jn = reinterpret_cast<double*>(base + oJn);
    tb.T = reinterpret_cast<float*>(base + oT);
    float2* Ca = reinterpret_cast<float2*>(base + oCa);
    float2* Cv = n_vox == 0 ? nullptr : reinterpret_cast<float2*>(base + oCv);
    DPX_CUDA(cudaMemsetAsync(Ca, 0, cell_set * (n_vox == 0 ? 1 : 2), st));
    // the side stream: the tables, then the atoms' set, beside the binning and
    // the voxels' moments (the voxels' contractions wait for aux_done, the
    // synthesis for aux_atoms)
    if (!ctx->aux) DPX_CUDA(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&ctx->aux_go, &ctx->aux_done, &ctx->aux_atoms})
        if (!*e) DPX_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    cudaStream_t ax = ctx->aux;
    DPX_CUDA(cudaEventRecord(ctx->aux_go, st));
    // from here on every return joins the side stream back into st, so that a
    // later call's staging on st cannot overwrite the arena while the tables or
    // the atoms' set still use it
    struct JoinAux {
        cudaStream_t st, ax;
        cudaEvent_t ev;
        bool joined = false;
        ~JoinAux() {
            if (joined) return;
            if (cudaEventRecord(ev, ax) == cudaSuccess) cudaStreamWaitEvent(st, ev, 0);
        }
    } join{st, ax, ctx->aux_atoms};
    DPX_CUDA(cudaStreamWaitEvent(ax, ctx->aux_go, 0));
    DPX_CUDA(dpx::launch_harmonic_tables(ax, tb));
    DPX_CUDA(cudaEventRecord(ctx->aux_done, ax));
    auto launch_set = [&](int k) -> int {
        const Set& S = *sets[k];
        if (S.units.empty()) return DPX_OK;
        dpx::HarmonicSet a{};
        a.pts = k == 0 ? reinterpret_cast<const float4*>(base + oP[0]) : vox_dev;
        a.units = reinterpret_cast<const int4*>(base + oU[k]);
        a.n_units = (int)S.units.size();
        a.groups = reinterpret_cast<const int2*>(base + oG[k]);
        a.gu = reinterpret_cast<const int*>(base + oGu[k]);
        a.G = (int)S.groups.size();
        a.LM = LM;
        a.K = K;
        a.Lp = Lp;
        a.nbins = nbins;
        a.delta = delta;
        a.ab = reinterpret_cast<const float2*>(base + oAb);
        a.cr = reinterpret_cast<const float2*>(base + oCr);
        a.nmm = reinterpret_cast<const float*>(base + oNm);
        a.T = tb.T;
        a.lmax = d_lmax;
        a.lmb = reinterpret_cast<const int*>(base + oLb);
        a.aff = reinterpret_cast<const float*>(dbase + t.aff);
        a.MP = reinterpret_cast<float2*>(base + (k == 0 ? oMPa : oMP));
        a.M = reinterpret_cast<float2*>(base + (k == 0 ? oMa : oM));
        a.ev0 = ev ? ev[2 * k] : nullptr;
        a.ev1 = ev ? ev[2 * k + 1] : nullptr;
        a.contract_wait = k == 0 ? nullptr : ctx->aux_done;  // the atoms run on the tables' stream
        DPX_CUDA(dpx::launch_harmonic_set(k == 0 ? ax : st, a, k == 0 ? Ca : Cv));
        return DPX_OK;
    };
    // ---- the voxels: their bin totals (the binning launched first) give the units ----
    if (n_vox) {
        if (int rc = bin_voxels_finish(ctx, nbins, sv.units, sv.groups, sv.gu)) return rc;
        if (sv.units.size() > vox_units_max || sv.groups.size() > (size_t)nbins)
            return fail(DPX_ERR_ARG, "harmonic fill: %zu voxel units above the %zu planned", sv.units.size(),
                        vox_units_max);
        const size_t bytes = oJn - oU[1];
        char* vp = nullptr;
        DPX_CUDA(ctx->pin_units.get(bytes, &vp));
        std::memcpy(vp, sv.units.data(), sv.units.size() * sizeof(int4));
        std::memcpy(vp + (oG[1] - oU[1]), sv.groups.data(), sv.groups.size() * sizeof(int2));
        std::memcpy(vp + (oGu[1] - oU[1]), sv.gu.data(), sv.gu.size() * sizeof(int));
        DPX_CUDA(cudaMemcpyAsync(base + oU[1], vp, bytes, cudaMemcpyHostToDevice, st));
        DPX_CUDA(ctx->pin_units.copied(st));
        if (int rc = launch_set(1)) return rc;
    }
    // ---- the atoms, grouped by (bin, ion) while the voxels' moments run ----
    make_set(centred_atoms(), false, sa);
    if (sa.units.size() > atom_units_max || sa.groups.size() > atom_groups_max)
        return fail(DPX_ERR_ARG, "harmonic fill: %zu atom units above the %zu planned", sa.units.size(),
                    atom_units_max);
    if (!sa.units.empty()) {
        const size_t bytes = oJn - oP[0];
        char* ap = nullptr;
        DPX_CUDA(ctx->pin_atomset.get(bytes, &ap));
        std::memcpy(ap, sa.pts.data(), sa.pts.size() * sizeof(float4));
        std::memcpy(ap + (oU[0] - oP[0]), sa.units.data(), sa.units.size() * sizeof(int4));
        std::memcpy(ap + (oG[0] - oP[0]), sa.groups.data(), sa.groups.size() * sizeof(int2));
        std::memcpy(ap + (oGu[0] - oP[0]), sa.gu.data(), sa.gu.size() * sizeof(int));
        DPX_CUDA(cudaMemcpyAsync(base + oP[0], ap, bytes, cudaMemcpyHostToDevice, ax));
        DPX_CUDA(ctx->pin_atomset.copied(ax));
        if (int rc = launch_set(0)) return rc;
    }
    DPX_CUDA(cudaEventRecord(ctx->aux_atoms, ax));
    DPX_CUDA(cudaStreamWaitEvent(st, ctx->aux_atoms, 0));
    join.joined = true;
    // F(0) with the solvent boxes' volumes, summed while the moments run
    const double origin = t.origin + d.scale * box_volume_sum(d);
    if (ev) {
        ctx->tev_used = n_vox ? 8 : 6;
        // K per point as the moments compute it: its bin's (l_b + 1)(l_b + 2) / 2
        double pk = 0.0;
        for (const Set* S : {&sa, &sv})
            for (const int4& u : S->units) pk += (double)u.y * (lmb[u.z] + 1) * (lmb[u.z] + 2) / 2;
        ctx->stage_points = (double)sa.pts.size() + (double)n_vox;
        ctx->stage_k = ctx->stage_points > 0 ? pk / ctx->stage_points : 0.0;
    }
    dpx::HarmonicSynth y{};
    y.Ca = Ca;
    y.Cv = Cv;
    y.K = K;
    y.Lp = Lp;
    y.lmax_host_outer = LM;
    y.lmax = d_lmax;
    y.ab = reinterpret_cast<const float2*>(base + oAb);
    y.nmm = reinterpret_cast<const float*>(base + oNm);
    y.step = G.step;
    y.vox_s = (float)s;
    y.cx = t.cen[0];
    y.cy = t.cen[1];
    y.cz = t.cen[2];
    y.use_center = (t.cen[0] != 0.0 || t.cen[1] != 0.0 || t.cen[2] != 0.0);
    y.scale = (float)d.scale;
    y.origin = origin;
    y.grid = reinterpret_cast<float4*>(grid);
    if (ev) DPX_CUDA(cudaEventRecord(ev[4], st));
    DPX_CUDA(dpx::launch_harmonic_synth(st, y));
    if (ev) {
        DPX_CUDA(cudaEventRecord(ev[5], st));
        DPX_CUDA(cudaEventRecord(ev[7], st));
    }
    // the arena and the pinned staging stay owned by the context
    return DPX_OK;
}

}  // namespace dpxh
