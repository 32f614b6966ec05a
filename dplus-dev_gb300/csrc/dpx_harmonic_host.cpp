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

// Basis table of a chunk kept under this many bytes, so that it stays in the
// 129 MB L2 while the GEMM re-reads it once per tile of shells.
constexpr size_t kChunkBasisBytes = size_t(80) << 20;

}  // namespace

int harmonic_fill(dpx_ctx ctx, const dpx_pdb_desc& d, const LeafTables& t, const char* dbase, const dpx::Geom& G,
                  void* grid) {
    const int Lp = G.Lp;
    if (t.n_boxes > 0 && !(d.voxel_step > 0.0)) return 1;
    // ---- point sets about the leaf's centre t.cen (device atoms arrive shifted) ----
    const float* src = d.atoms;
    std::vector<float> dev_copy;
    if (d.atoms_on_device) {
        dev_copy.resize((size_t)4 * d.n_atoms);
        DPX_CUDA(cudaMemcpyAsync(dev_copy.data(), d.atoms, dev_copy.size() * sizeof(float), cudaMemcpyDeviceToHost,
                                 ctx->stream));
        DPX_CUDA(cudaStreamSynchronize(ctx->stream));
        src = dev_copy.data();
    }
    const double sh[3] = {d.atoms_on_device ? 0.0 : t.cen[0], d.atoms_on_device ? 0.0 : t.cen[1],
                          d.atoms_on_device ? 0.0 : t.cen[2]};
    std::vector<float4> atoms(d.n_atoms);
    {
        int64_t j = 0;
        for (int u = 0; u < d.n_ions; ++u)
            for (int k = 0; k < d.atoms_per_ion[u]; ++k, ++j)
                atoms[j] = make_float4((float)((double)src[4 * j] - sh[0]), (float)((double)src[4 * j + 1] - sh[1]),
                                       (float)((double)src[4 * j + 2] - sh[2]), (float)u);
    }
    std::vector<float4> vox;
    const double s = d.voxel_step;
    if (t.n_boxes > 0) {
        for (int64_t b = 0; b < t.n_boxes; ++b) {
            const float* r = d.boxes + 8 * b;
            const int nx = (int)std::lround(r[4] / s), ny = (int)std::lround(r[5] / s), nz = (int)std::lround(r[6] / s);
            for (int ix = 0; ix < nx; ++ix)
                for (int iy = 0; iy < ny; ++iy)
                    for (int iz = 0; iz < nz; ++iz)
                        vox.push_back(make_float4(
                            (float)((double)r[0] + ((ix + 0.5) * s - 0.5 * r[4]) - t.cen[0]),
                            (float)((double)r[1] + ((iy + 0.5) * s - 0.5 * r[5]) - t.cen[1]),
                            (float)((double)r[2] + ((iz + 0.5) * s - 0.5 * r[6]) - t.cen[2]), r[3]));
        }
    }
    double R = 0.0;
    for (const float4& p : atoms) R = std::max(R, std::sqrt((double)p.x * p.x + (double)p.y * p.y + (double)p.z * p.z));
    for (const float4& p : vox) R = std::max(R, std::sqrt((double)p.x * p.x + (double)p.y * p.y + (double)p.z * p.z));
    // ---- orders ----
    std::vector<int> lmax(Lp + 1, 0);
    for (int i = 1; i <= Lp; ++i) lmax[i] = order_of(i * G.step * R);
    const int LM = lmax[Lp];
    if (LM > dpx::harmonic_max_l()) return 1;
    const int K = (LM + 1) * (LM + 2) / 2;
    std::vector<int> imin(LM + 1, Lp + 1);
    for (int l = 0; l <= LM; ++l)
        for (int i = 1; i <= Lp; ++i)
            if (lmax[i] >= l) {
                imin[l] = i;
                break;
            }
    std::vector<int64_t> joff(LM + 1, 0);
    int64_t rows_total = 0;
    for (int l = 0; l <= LM; ++l) {
        joff[l] = rows_total;
        rows_total += Lp - imin[l] + 1;
    }
    std::vector<float2> ab(K, make_float2(0.f, 0.f));
    for (int m = 0; m <= LM; ++m)
        for (int l = m + 1; l <= LM; ++l) {
            const double a = std::sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            const double b = std::sqrt((((double)l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
            ab[(size_t)l * (l + 1) / 2 + m] = make_float2((float)a, (float)b);
        }
    std::vector<int2> rows;
    for (int i = 1; i <= Lp; ++i)
        for (int tt = 0; tt <= 3 * i / 2; ++tt) rows.push_back(make_int2(i, tt));
    // ---- chunking ----
    const int64_t npts = std::max<int64_t>((int64_t)atoms.size(), (int64_t)vox.size());
    int64_t ch = (int64_t)(kChunkBasisBytes / ((size_t)K * sizeof(float2))) / 64 * 64;
    ch = std::max<int64_t>(64, std::min<int64_t>(ch, (npts + 63) / 64 * 64));
    const size_t cell_set = (size_t)(Lp + 1) * K * sizeof(double2);
    // ---- device arena ----
    std::vector<char> h;
    const size_t oA = put(h, atoms.data(), atoms.size() * sizeof(float4));
    const size_t oV = put(h, vox.data(), vox.size() * sizeof(float4));
    const size_t oL = put(h, lmax.data(), lmax.size() * sizeof(int));
    const size_t oI = put(h, imin.data(), imin.size() * sizeof(int));
    const size_t oJo = put(h, joff.data(), joff.size() * sizeof(int64_t));
    const size_t oAb = put(h, ab.data(), ab.size() * sizeof(float2));
    const size_t oR = put(h, rows.data(), rows.size() * sizeof(int2));
    const size_t staged = al16(h.size());
    const size_t oY = staged;
    const size_t oJ = al16(oY + (size_t)K * ch * sizeof(float2));
    const size_t oCa = al16(oJ + (size_t)rows_total * ch * sizeof(float));
    const size_t oCv = al16(oCa + cell_set);
    const size_t total = oCv + (vox.empty() ? 0 : cell_set);
    if (cudaError_t e = ctx->harmonic.reserve(total)) {
        cudaGetLastError();
        return fail(DPX_ERR_OOM, "harmonic fill needs %zu bytes (%s)", total, cudaGetErrorString(e));
    }
    char* base = static_cast<char*>(ctx->harmonic.p);
    cudaStream_t st = ctx->stream;
    DPX_CUDA(cudaMemcpyAsync(base, h.data(), staged, cudaMemcpyHostToDevice, st));
    dpx::HarmonicArgs a{};
    a.ch = (int)ch;
    a.Lp = Lp;
    a.LM = LM;
    a.K = K;
    a.step = G.step;
    a.lmax = reinterpret_cast<const int*>(base + oL);
    a.imin = reinterpret_cast<const int*>(base + oI);
    a.joff = reinterpret_cast<const int64_t*>(base + oJo);
    a.ab = reinterpret_cast<const float2*>(base + oAb);
    a.aff = reinterpret_cast<const float*>(dbase + t.aff);
    a.Y = reinterpret_cast<float2*>(base + oY);
    a.J = reinterpret_cast<float*>(base + oJ);
    double2* Ca = reinterpret_cast<double2*>(base + oCa);
    double2* Cv = vox.empty() ? nullptr : reinterpret_cast<double2*>(base + oCv);
    DPX_CUDA(cudaMemsetAsync(Ca, 0, cell_set * (vox.empty() ? 1 : 2), st));
    for (int set = 0; set < 2; ++set) {
        const bool voxels = set == 1;
        const int64_t n = voxels ? (int64_t)vox.size() : (int64_t)atoms.size();
        if (n == 0) continue;
        a.pts = reinterpret_cast<const float4*>(base + (voxels ? oV : oA));
        a.n = n;
        const int64_t nc = (n + ch - 1) / ch;
        for (int64_t c = 0; c < nc; ++c)
            DPX_CUDA(dpx::launch_harmonic_chunk(st, a, voxels, c * ch, voxels ? Cv : Ca));
    }
    dpx::HarmonicSynth y{};
    y.rows = reinterpret_cast<const int2*>(base + oR);
    y.n_rows = (int)rows.size();
    y.Ca = Ca;
    y.Cv = Cv;
    y.K = K;
    y.Lp = Lp;
    y.lmax_host_outer = LM;
    y.lmax = a.lmax;
    y.ab = a.ab;
    y.step = G.step;
    y.vox_s = (float)s;
    y.cx = t.cen[0];
    y.cy = t.cen[1];
    y.cz = t.cen[2];
    y.use_center = (t.cen[0] != 0.0 || t.cen[1] != 0.0 || t.cen[2] != 0.0);
    y.scale = (float)d.scale;
    y.origin = t.origin;
    y.grid = reinterpret_cast<float4*>(grid);
    DPX_CUDA(dpx::launch_harmonic_synth(st, y));
    // the staging vectors are host-side; the copy above was from pageable
    // memory and has completed, the arena stays owned by the context
    return DPX_OK;
}

}  // namespace dpxh
