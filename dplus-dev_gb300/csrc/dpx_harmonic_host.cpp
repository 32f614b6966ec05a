// dpx_harmonic_host.cpp — planning and launching of the harmonic FP32 fill
// (dpx_harmonic.cu) of one leaf.
//
// harmonic_plan does everything that needs the host or a synchronization, once
// per leaf and grid geometry: the radius of the point sets about the leaf's
// centre (which sets the expansion orders), the solvent boxes expanded into
// voxels and sorted by radial bin on the device, the atoms grouped by (bin,
// ion) on the host, the units of <= kUnitPoints points, the recurrence tables
// and the form factors, all copied into a device arena the plan owns.
// harmonic_launch then queues kernels only (no host work, no copies from the
// host, no synchronization), so the fill can be recorded in a CUDA graph and
// replayed; its scratch comes from the caller.
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

// Stream-ordered device scratch of the planning, freed on its stream when it
// goes out of scope (after the work queued on it).
struct TmpDev {
    cudaStream_t s;
    void* p = nullptr;
    explicit TmpDev(cudaStream_t st) : s(st) {}
    ~TmpDev() {
        if (p) cudaFreeAsync(p, s);
    }
    cudaError_t get(size_t n) { return cudaMallocAsync(&p, n ? n : 16, s); }
};

struct Set {
    std::vector<float4> pts;
    std::vector<int4> units;
    std::vector<int2> groups;
    std::vector<int> gu;
};

// Points grouped by (bin, ion) for atoms (w = ion index) in a stable counting
// sort, units of <= kUnitPoints points per group.
void make_atom_set(const std::vector<float4>& in, int n_ions, int nbins, double delta, Set& out) {
    const int ng = nbins * n_ions;
    std::vector<int> gid(in.size()), count(ng + 1, 0);
    for (size_t j = 0; j < in.size(); ++j) {
        const float4& p = in[j];
        const double r = std::sqrt((double)p.x * p.x + (double)p.y * p.y + (double)p.z * p.z);
        const int b = std::min(nbins - 1, (int)(r / delta));
        gid[j] = b * n_ions + (int)p.w;
        count[gid[j] + 1]++;
    }
    for (int g = 0; g < ng; ++g) count[g + 1] += count[g];
    out.pts.resize(in.size());
    std::vector<int> fill(count.begin(), count.end() - 1);
    for (size_t j = 0; j < in.size(); ++j) {
        float4 p = in[j];
        p.w = 1.f;  // the ion's form factor is applied per shell
        out.pts[fill[gid[j]]++] = p;
    }
    for (int g = 0; g < ng; ++g) {
        const int n = count[g + 1] - count[g];
        if (n == 0) continue;
        out.gu.push_back((int)out.units.size());
        out.groups.push_back(make_int2(g / n_ions, g % n_ions));
        for (int o = 0; o < n; o += kUnitPoints)
            out.units.push_back(make_int4(count[g] + o, std::min(kUnitPoints, n - o), g / n_ions, 0));
    }
    out.gu.push_back((int)out.units.size());
}

// The tensor-core moments' CTAs of a set: units[].w = the unit's first CTA
// (dpx::tc_parts of its bin's order per unit); returns the set's total.
int number_parts(std::vector<int4>& units, const std::vector<int>& lmb) {
    int n = 0;
    for (int4& u : units) {
        u.w = n;
        n += dpx::tc_parts(lmb[u.z]);
    }
    return n;
}

}  // namespace

int harmonic_plan(cudaStream_t st, const dpx_pdb_desc& d, const dpx::Geom& G, HarmPlan& p) {
    p = HarmPlan{};
    p.G = G;
    p.stream = st;
    if (d.n_boxes > 0 && d.boxes && !(d.voxel_step > 0.0)) return kHarmDeclined;
    // ---- the atoms on the host (device atoms arrive shifted by the centre) ----
    std::vector<float> host_atoms;
    const float* src = d.atoms;
    if (d.atoms_on_device) {
        host_atoms.resize((size_t)4 * d.n_atoms);
        DPX_CUDA(cudaMemcpyAsync(host_atoms.data(), d.atoms, host_atoms.size() * sizeof(float),
                                 cudaMemcpyDeviceToHost, st));
        DPX_CUDA(cudaStreamSynchronize(st));
        src = host_atoms.data();
    }
    // the centre restored per cell: the given one, else the host atoms' centroid
    // (as stage_leaf centres FP32 grids)
    double c[3] = {0, 0, 0};
    if (d.center) {
        for (int k = 0; k < 3; ++k) c[k] = d.center[k];
    } else if (!d.atoms_on_device) {
        for (int64_t a = 0; a < d.n_atoms; ++a)
            for (int k = 0; k < 3; ++k) c[k] += src[4 * a + k];
        for (int k = 0; k < 3; ++k) c[k] /= (double)d.n_atoms;
    }
    for (int k = 0; k < 3; ++k) p.cen[k] = c[k];
    const double sh[3] = {d.atoms_on_device ? 0.0 : c[0], d.atoms_on_device ? 0.0 : c[1],
                          d.atoms_on_device ? 0.0 : c[2]};
    std::vector<float4> atoms(d.n_atoms);
    double r2 = 0.0;
    {
        int64_t j = 0;
        for (int u = 0; u < d.n_ions; ++u)
            for (int k = 0; k < d.atoms_per_ion[u]; ++k, ++j) {
                atoms[j] = make_float4((float)((double)src[4 * j] - sh[0]), (float)((double)src[4 * j + 1] - sh[1]),
                                       (float)((double)src[4 * j + 2] - sh[2]), (float)u);
                double q = 0;
                for (int a = 0; a < 3; ++a) q += ((double)src[4 * j + a] - sh[a]) * ((double)src[4 * j + a] - sh[a]);
                r2 = std::max(r2, q);
            }
    }
    double r2_pts = r2;  // the points themselves: atoms and voxel centres
    // ---- the solvent boxes: centred and counted on the device, with their
    // largest corner and voxel-centre distances and the voxel total ----
    const int64_t nb = d.n_boxes > 0 && d.boxes ? d.n_boxes : 0;
    TmpDev tboxes(st);
    dpx::VoxelPrepArgs pa{};
    size_t oVs = 0, oRs = 0;
    int64_t nv = 0;
    if (nb > 0) {
        const size_t oRaw = 0;
        const size_t oBox = al16((size_t)8 * nb * sizeof(float));
        const size_t oCnt = al16(oBox + (size_t)2 * nb * sizeof(float4));
        oVs = al16(oCnt + (size_t)nb * sizeof(int64_t));
        oRs = al16(oVs + (size_t)nb * sizeof(int64_t));
        const size_t oSc = al16(oRs + (size_t)((nb + dpx::kVoxelScanRun - 1) / dpx::kVoxelScanRun) * sizeof(int64_t));
        DPX_CUDA(tboxes.get(oSc + 3 * sizeof(unsigned long long)));
        char* base = static_cast<char*>(tboxes.p);
        DPX_CUDA(cudaMemcpyAsync(base + oRaw, d.boxes, (size_t)8 * nb * sizeof(float), cudaMemcpyHostToDevice, st));
        pa.raw = reinterpret_cast<const float*>(base + oRaw);
        pa.nb = nb;
        pa.cx = c[0];
        pa.cy = c[1];
        pa.cz = c[2];
        pa.vs = (float)d.voxel_step;
        pa.boxes = reinterpret_cast<float4*>(base + oBox);
        pa.counts = reinterpret_cast<int64_t*>(base + oCnt);
        pa.scal = reinterpret_cast<unsigned long long*>(base + oSc);
        DPX_CUDA(dpx::launch_voxel_prepare(st, pa));
        unsigned long long sc[3];
        DPX_CUDA(cudaMemcpyAsync(sc, pa.scal, sizeof sc, cudaMemcpyDeviceToHost, st));
        DPX_CUDA(cudaStreamSynchronize(st));
        const unsigned qbits = (unsigned)sc[0], vbits = (unsigned)sc[2];
        float qf, vf;
        std::memcpy(&qf, &qbits, sizeof qf);
        std::memcpy(&vf, &vbits, sizeof vf);
        r2_pts = std::max(r2_pts, (double)vf);
        r2 = std::max(r2, (double)qf);
        nv = (int64_t)sc[1];
        if (nv > INT32_MAX) return fail(DPX_ERR_ARG, "harmonic fill: %lld voxels", (long long)nv);
    }
    // ---- orders and radial bins; leaves beyond the kernels' limits decline ----
    const int Lp = G.Lp;
    const double R = std::sqrt(r2) * (1.0 + 1e-6);  // the points are rounded to FP32 about the centre
    // R bounds the atoms and the box corners (and so the bins), Reff the atoms
    // and the voxel centres (and so the orders); bin b needs the orders
    // l <= order_of(q_max (b + 1) delta) only
    const double Reff = std::min(R, std::sqrt(r2_pts) * (1.0 + 1e-6));
    if (order_of(Lp * G.step * R) > dpx::harmonic_max_l()) return kHarmDeclined;
    const double delta = kBinWidthTimesQmax / (Lp * G.step);
    const int nbins = (int)(R / delta) + 1;
    if (nb > 0 && nbins > dpx::harmonic_max_bins()) return kHarmDeclined;
    std::vector<int> lmax(Lp + 1, 0);
    for (int i = 1; i <= Lp; ++i) lmax[i] = order_of(i * G.step * Reff);
    const int LM = lmax[Lp];
    if (LM > dpx::harmonic_max_l()) return kHarmDeclined;
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
            const double cc = l >= m + 2 ? 4.0 * b / a_prev : 0.0;
            cr[(size_t)l * (l + 1) / 2 + m] = make_float2((float)cc, (float)r);
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
    double nodes[6], vinv[36];
    chebyshev_fit(nodes, vinv);
    std::vector<double> affd;
    leaf_aff_table(d, Lp, G.step, affd);
    std::vector<float> aff(affd.begin(), affd.end());
    double origin = 0.0;  // F(0): the form factors at shell 0 times the ion counts, plus the box volumes
    for (int u = 0; u < d.n_ions; ++u) origin += affd[(size_t)u * (Lp + 1)] * d.atoms_per_ion[u];
    origin += box_volume_sum(d);
    // ---- the atoms grouped by (bin, ion) ----
    Set sa;
    make_atom_set(atoms, d.n_ions, nbins, delta, sa);
    // ---- the device arena: tables, the atoms' set, the voxels (binned below) ----
    p.n_parts[0] = number_parts(sa.units, lmb);
    std::vector<char> h;
    p.o_lmax = put(h, lmax.data(), lmax.size() * sizeof(int));
    p.o_lmb = put(h, lmb.data(), lmb.size() * sizeof(int));
    p.o_ab = put(h, ab.data(), ab.size() * sizeof(float2));
    p.o_cr = put(h, cr.data(), cr.size() * sizeof(float2));
    p.o_nmm = put(h, nmm.data(), nmm.size() * sizeof(float));
    p.o_nodes = put(h, nodes, sizeof nodes);
    p.o_vinv = put(h, vinv, sizeof vinv);
    p.o_aff = put(h, aff.data(), aff.size() * sizeof(float));
    p.o_pts[0] = put(h, sa.pts.data(), sa.pts.size() * sizeof(float4));
    p.o_units[0] = put(h, sa.units.data(), sa.units.size() * sizeof(int4));
    p.o_groups[0] = put(h, sa.groups.data(), sa.groups.size() * sizeof(int2));
    p.o_gu[0] = put(h, sa.gu.data(), sa.gu.size() * sizeof(int));
    const size_t staged = al16(h.size());
    // the voxels' set: units and groups after the bin totals, the points binned on the device
    const size_t vox_units_max = nv ? (size_t)(nv + kUnitPoints - 1) / kUnitPoints + nbins : 0;
    p.o_units[1] = staged;
    p.o_groups[1] = al16(p.o_units[1] + vox_units_max * sizeof(int4));
    p.o_gu[1] = al16(p.o_groups[1] + (size_t)nbins * sizeof(int2));
    p.o_pts[1] = al16(p.o_gu[1] + (size_t)(nbins + 1) * sizeof(int));
    p.o_job = al16(nv ? p.o_pts[1] + (size_t)nv * sizeof(float4) : staged);
    // the radial tables T_n(i, b, l): they depend on the grid's shells and the
    // radial bins only, so they are computed here once, not in every fill
    p.o_T = al16(p.o_job + sizeof(dpx::HarmJob));
    p.arena_bytes = p.o_T + (size_t)(Lp + 1) * nbins * (LM + 1) * 8 * sizeof(float) + 16;
    DPX_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p.arena), p.arena_bytes, st));
    DPX_CUDA(cudaMemcpyAsync(p.arena, h.data(), staged, cudaMemcpyHostToDevice, st));
    {
        TmpDev jn(st);  // j_l at the nodes, FP64, freed in stream order after the fit
        DPX_CUDA(jn.get((size_t)(Lp + 1) * nbins * 6 * (LM + 1) * sizeof(double)));
        dpx::RadialTableArgs ra{};
        ra.Lp = Lp;
        ra.nbins = nbins;
        ra.LM = LM;
        ra.step = G.step;
        ra.delta = delta;
        ra.lmax = reinterpret_cast<const int*>(p.arena + p.o_lmax);
        ra.nodes = reinterpret_cast<const double*>(p.arena + p.o_nodes);
        ra.vinv = reinterpret_cast<const double*>(p.arena + p.o_vinv);
        ra.Jn = static_cast<double*>(jn.p);
        ra.T = reinterpret_cast<float*>(p.arena + p.o_T);
        DPX_CUDA(dpx::launch_radial_tables(st, ra));
    }
    // ---- the voxels: expanded and sorted by bin on the device, units from the totals ----
    Set sv;
    if (nv > 0) {
        const int nblk = (int)((nv + 255) / 256);
        const size_t oTmp = 0;
        const size_t oBin = al16(oTmp + (size_t)nv * sizeof(float4));
        const size_t oHist = al16(oBin + (size_t)nv * sizeof(int));
        const size_t oOff = al16(oHist + (size_t)nbins * nblk * sizeof(int));
        const size_t oTot = al16(oOff + (size_t)nbins * nblk * sizeof(int64_t));
        TmpDev tbin(st);
        DPX_CUDA(tbin.get(oTot + (size_t)nbins * sizeof(int64_t)));
        char* base = static_cast<char*>(tbin.p);
        char* tb = static_cast<char*>(tboxes.p);
        dpx::VoxelBinArgs a{};
        a.boxes = pa.boxes;
        a.counts = pa.counts;
        a.vstart = reinterpret_cast<int64_t*>(tb + oVs);
        a.run_sums = reinterpret_cast<int64_t*>(tb + oRs);
        a.nb = nb;
        a.nv = nv;
        a.vs = (float)d.voxel_step;
        a.delta = (float)delta;
        a.nbins = nbins;
        a.tmp = reinterpret_cast<float4*>(base + oTmp);
        a.vbin = reinterpret_cast<int*>(base + oBin);
        a.hist = reinterpret_cast<int*>(base + oHist);
        a.off = reinterpret_cast<int64_t*>(base + oOff);
        a.total = reinterpret_cast<int64_t*>(base + oTot);
        a.out = reinterpret_cast<float4*>(p.arena + p.o_pts[1]);
        DPX_CUDA(dpx::launch_voxel_bins(st, a));
        std::vector<int64_t> tot(nbins);
        DPX_CUDA(cudaMemcpyAsync(tot.data(), a.total, (size_t)nbins * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        DPX_CUDA(cudaStreamSynchronize(st));
        int64_t start = 0;
        for (int bin = 0; bin < nbins; ++bin) {
            const int64_t cnt = tot[bin];
            if (cnt > 0) {
                sv.gu.push_back((int)sv.units.size());
                sv.groups.push_back(make_int2(bin, -1));
                for (int64_t o = 0; o < cnt; o += kUnitPoints)
                    sv.units.push_back(
                        make_int4((int)(start + o), (int)std::min<int64_t>(kUnitPoints, cnt - o), bin, 0));
            }
            start += cnt;
        }
        sv.gu.push_back((int)sv.units.size());
        p.n_parts[1] = number_parts(sv.units, lmb);
        if (sv.units.size() > vox_units_max || start != nv)
            return fail(DPX_ERR_ARG, "harmonic fill: %zu voxel units above the %zu planned", sv.units.size(),
                        vox_units_max);
        std::vector<char> hv(p.o_pts[1] - p.o_units[1]);
        std::memcpy(hv.data(), sv.units.data(), sv.units.size() * sizeof(int4));
        std::memcpy(hv.data() + (p.o_groups[1] - p.o_units[1]), sv.groups.data(), sv.groups.size() * sizeof(int2));
        std::memcpy(hv.data() + (p.o_gu[1] - p.o_units[1]), sv.gu.data(), sv.gu.size() * sizeof(int));
        DPX_CUDA(cudaMemcpyAsync(p.arena + p.o_units[1], hv.data(), hv.size(), cudaMemcpyHostToDevice, st));
        // the pageable source must stay valid until its copy is done
        DPX_CUDA(cudaStreamSynchronize(st));
    }
    DPX_CUDA(dpx::harmonic_reserve_smem(Lp, LM));
    // ---- the plan's figures and the scratch layout of a launch ----
    p.nbins = nbins;
    p.LM = LM;
    p.K = K;
    p.delta = delta;
    p.n_vox = nv;
    p.n_units[0] = (int)sa.units.size();
    p.n_groups[0] = (int)sa.groups.size();
    p.n_units[1] = (int)sv.units.size();
    p.n_groups[1] = (int)sv.groups.size();
    p.scale = (float)d.scale;
    p.origin = origin * d.scale;
    p.vox_s = (float)d.voxel_step;
    double pk = 0.0;  // K per point as the moments compute it: its bin's (l_b + 1)(l_b + 2) / 2
    for (const Set* S : {&sa, &sv})
        for (const int4& u : S->units) pk += (double)u.y * (lmb[u.z] + 1) * (lmb[u.z] + 2) / 2;
    p.stage_points = (double)sa.pts.size() + (double)nv;
    p.stage_k = p.stage_points > 0 ? pk / p.stage_points : 0.0;
    const size_t cell_set = (size_t)(Lp + 1) * K * sizeof(float2);
    const size_t mpu = (size_t)6 * K * sizeof(float2);  // moments of a unit or a group
    size_t o = 0;
    auto take = [&](size_t n) {
        const size_t at = (o + 255) & ~size_t(255);
        o = at + n;
        return at;
    };
    for (int k = 0; k < 2; ++k) {
        p.s_MP[k] = take((size_t)p.n_units[k] * mpu);
        p.s_M[k] = take((size_t)p.n_groups[k] * mpu);
    }
    p.s_C[0] = take(cell_set);
    p.s_C[1] = take(nv ? cell_set : 0);
    p.scratch_bytes = o + 256;
    // the plan's own job: its scratch and grid at the launch's bases
    dpx::HarmJob job = harmonic_job(p, 0, 0);
    p.shape = dpx::plan_harmonic_jobs(&job, 1);
    DPX_CUDA(cudaMemcpyAsync(p.arena + p.o_job, &job, sizeof job, cudaMemcpyHostToDevice, st));
    // the pageable staging above must stay valid until its copy is done
    DPX_CUDA(cudaStreamSynchronize(st));
    return DPX_OK;
}

void harmonic_plan_release(HarmPlan& p) {
    if (p.arena) cudaFreeAsync(p.arena, p.stream);
    p.arena = nullptr;
    p.arena_bytes = 0;
}

dpx::HarmJob harmonic_job(const HarmPlan& p, size_t scratch_off, size_t grid_off) {
    const char* base = p.arena;
    dpx::HarmJob J{};
    J.Lp = p.G.Lp;
    J.nbins = p.nbins;
    J.LM = p.LM;
    J.K = p.K;
    J.step = p.G.step;
    J.delta = p.delta;
    J.lmax = reinterpret_cast<const int*>(base + p.o_lmax);
    J.lmb = reinterpret_cast<const int*>(base + p.o_lmb);
    J.nodes = reinterpret_cast<const double*>(base + p.o_nodes);
    J.vinv = reinterpret_cast<const double*>(base + p.o_vinv);
    J.ab = reinterpret_cast<const float2*>(base + p.o_ab);
    J.cr = reinterpret_cast<const float2*>(base + p.o_cr);
    J.nmm = reinterpret_cast<const float*>(base + p.o_nmm);
    J.aff = reinterpret_cast<const float*>(base + p.o_aff);
    for (int k = 0; k < 2; ++k) {
        J.pts[k] = reinterpret_cast<const float4*>(base + p.o_pts[k]);
        J.units[k] = reinterpret_cast<const int4*>(base + p.o_units[k]);
        J.groups[k] = reinterpret_cast<const int2*>(base + p.o_groups[k]);
        J.gu[k] = reinterpret_cast<const int*>(base + p.o_gu[k]);
        J.n_units[k] = p.n_units[k];
        J.n_parts[k] = p.n_parts[k];
        J.G[k] = p.n_groups[k];
        J.s_MP[k] = scratch_off + p.s_MP[k];
        J.s_M[k] = scratch_off + p.s_M[k];
        J.s_C[k] = scratch_off + p.s_C[k];
    }
    J.vox = p.n_vox > 0;
    J.use_center = (p.cen[0] != 0.0 || p.cen[1] != 0.0 || p.cen[2] != 0.0);
    J.vox_s = p.vox_s;
    J.scale = p.scale;
    J.cx = p.cen[0];
    J.cy = p.cen[1];
    J.cz = p.cen[2];
    J.origin = p.origin;
    J.T = reinterpret_cast<const float*>(base + p.o_T);
    J.grid_off = grid_off;
    return J;
}

int harmonic_launch(const HarmStreams& S, const HarmPlan& p, void* scratch, float4* grid) {
    if (!p.arena) return fail(DPX_ERR_ARG, "harmonic fill: no plan");
    cudaEvent_t* ev = S.tev;  // [0, 1] moments, [4, 5] synthesis, [6, 7] the whole fill
    cudaEvent_t stage[4] = {ev ? ev[0] : nullptr, ev ? ev[1] : nullptr, ev ? ev[4] : nullptr, ev ? ev[5] : nullptr};
    if (ev) DPX_CUDA(cudaEventRecord(ev[6], S.st));
    DPX_CUDA(dpx::launch_harmonic_jobs(S.st, reinterpret_cast<const dpx::HarmJob*>(p.arena + p.o_job), 1, p.shape,
                                       static_cast<char*>(scratch), reinterpret_cast<char*>(grid), stage));
    if (ev) DPX_CUDA(cudaEventRecord(ev[7], S.st));
    return DPX_OK;
}

int harmonic_launches(const HarmPlan& p) {
    const dpx::HarmShape& h = p.shape;
    return (h.moments > 0) + (h.groups > 0) + (h.contract > 0) + (h.synth > 0);
}

}  // namespace dpxh
