// dpx_stage.cpp — staging of one PDB leaf's device tables for the amplitude
// fill, shared by the single/batched fill, the batched solves and the server:
// centred float4 atoms, ion offsets, the form-factor table, the work-item
// prefix and the voxelized-solvent boxes, appended to a host byte buffer that
// is copied to the device in one piece.
#include "dpx_host.h"

#include <algorithm>
#include <cstring>

namespace dpxh {

namespace {
size_t put(std::vector<char>& h, const void* src, size_t n) {
    const size_t at = al16(h.size());
    h.resize(at + n);
    if (n && src) std::memcpy(h.data() + at, src, n);
    return at;
}
}  // namespace

void stage_leaf(std::vector<char>& h, const dpx_pdb_desc& d, const dpx::Geom& G, bool fp32, int cpt, LeafTables& t,
                bool direct_boxes) {
    // centring: FP32 grids shift host atoms by the given centre or their
    // centroid, restored per cell as e^{i q.c}; FP64 grids take host atoms as
    // they are; device atoms arrive already shifted by the given centre
    for (int k = 0; k < 3; ++k) t.cen[k] = 0.0;
    if (d.center) {
        for (int k = 0; k < 3; ++k) t.cen[k] = d.center[k];
    } else if (!d.atoms_on_device && fp32) {
        double acc[3] = {0, 0, 0};
        for (int64_t a = 0; a < d.n_atoms; ++a)
            for (int k = 0; k < 3; ++k) acc[k] += d.atoms[4 * a + k];
        for (int k = 0; k < 3; ++k) t.cen[k] = acc[k] / double(d.n_atoms);
    }
    if (!fp32 && !d.atoms_on_device) t.cen[0] = t.cen[1] = t.cen[2] = 0.0;
    t.atoms = SIZE_MAX;
    if (!d.atoms_on_device) {
        t.atoms = put(h, nullptr, (size_t)d.n_atoms * sizeof(float4));
        float4* a = reinterpret_cast<float4*>(h.data() + t.atoms);
        for (int64_t i = 0; i < d.n_atoms; ++i)
            a[i] = make_float4((float)((double)d.atoms[4 * i] - t.cen[0]),
                               (float)((double)d.atoms[4 * i + 1] - t.cen[1]),
                               (float)((double)d.atoms[4 * i + 2] - t.cen[2]), 0.f);
    }
    std::vector<int> off(d.n_ions + 1, 0);
    for (int u = 0; u < d.n_ions; ++u) off[u + 1] = off[u] + d.atoms_per_ion[u];
    t.off = put(h, off.data(), off.size() * sizeof(int));
    std::vector<double> aff;
    leaf_aff_table(d, G.Lp, G.step, aff);
    if (fp32) {
        std::vector<float> af(aff.begin(), aff.end());
        t.aff = put(h, af.data(), af.size() * sizeof(float));
    } else {
        t.aff = put(h, aff.data(), aff.size() * sizeof(double));
    }
    double origin = 0.0;  // F(0): the form factors at shell 0 times the ion counts, plus the box volumes
    for (int u = 0; u < d.n_ions; ++u) origin += aff[(size_t)u * (G.Lp + 1)] * d.atoms_per_ion[u];
    std::vector<int64_t> pref(G.Lp + 1);
    t.items = dpx::fill_items(G, cpt, pref.data());
    t.pref = put(h, pref.data(), pref.size() * sizeof(int64_t));
    t.n_boxes = d.n_boxes > 0 && d.boxes ? d.n_boxes : 0;
    t.boxes = SIZE_MAX;
    if (t.n_boxes && direct_boxes) {  // {cx, cy, cz, w}, {Lx, Ly, Lz, 0}, centres shifted like the atoms
        // sorted by extent (as PrepareParametersForGPU sorts, PDBAmplitude.cpp:1351-1360) so
        // the fill recomputes its extent factors only where an extent changes
        std::vector<int64_t> order(t.n_boxes);
        for (int64_t i = 0; i < t.n_boxes; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
            const float* A = d.boxes + 8 * a + 4;
            const float* B = d.boxes + 8 * b + 4;
            if (A[0] != B[0]) return A[0] < B[0];
            if (A[1] != B[1]) return A[1] < B[1];
            return A[2] < B[2];
        });
        t.boxes = put(h, nullptr, (size_t)t.n_boxes * 2 * sizeof(float4));
        float4* b = reinterpret_cast<float4*>(h.data() + t.boxes);
        for (int64_t i = 0; i < t.n_boxes; ++i) {
            const float* s = d.boxes + 8 * order[i];
            b[2 * i] = make_float4((float)((double)s[0] - t.cen[0]), (float)((double)s[1] - t.cen[1]),
                                   (float)((double)s[2] - t.cen[2]), s[3]);
            b[2 * i + 1] = make_float4(s[4], s[5], s[6], 0.f);
        }
    }
    if (direct_boxes) origin += box_volume_sum(d);
    t.origin = origin * d.scale;
}

double box_volume_sum(const dpx_pdb_desc& d) {
    double v = 0.0;
    const int64_t nb = d.n_boxes > 0 && d.boxes ? d.n_boxes : 0;
    for (int64_t i = 0; i < nb; ++i) {
        const float* s = d.boxes + 8 * i;
        v += (double)s[3] * (double)s[4] * (double)s[5] * (double)s[6];
    }
    return v;
}

dpx::FillJob make_job(const dpx_pdb_desc& d, const LeafTables& t, const char* dbase, const dpx::Geom& G, void* grid,
                      int64_t tile_start) {
    dpx::FillJob J{};
    J.atoms = t.atoms == SIZE_MAX ? reinterpret_cast<const float4*>(d.atoms)
                                  : reinterpret_cast<const float4*>(dbase + t.atoms);
    J.ion_off = reinterpret_cast<const int*>(dbase + t.off);
    J.aff_f32 = reinterpret_cast<const float*>(dbase + t.aff);
    J.pref = reinterpret_cast<const int64_t*>(dbase + t.pref);
    J.boxes = t.n_boxes ? reinterpret_cast<const float4*>(dbase + t.boxes) : nullptr;
    J.n_boxes = (int)t.n_boxes;
    J.grid = reinterpret_cast<float4*>(grid);
    J.n_items = t.items;
    J.tile_start = tile_start;
    J.step = G.step;
    J.cx = t.cen[0];
    J.cy = t.cen[1];
    J.cz = t.cen[2];
    J.use_center = (t.cen[0] != 0.0 || t.cen[1] != 0.0 || t.cen[2] != 0.0);
    J.U = d.n_ions;
    J.Lp = G.Lp;
    J.scale = (float)d.scale;
    J.origin = t.origin;
    return J;
}

cudaError_t launch_leaf_f64(cudaStream_t s, const dpx_pdb_desc& d, const LeafTables& t, const char* dbase,
                            const dpx::Geom& G, void* grid) {
    const float4* atoms = t.atoms == SIZE_MAX ? reinterpret_cast<const float4*>(d.atoms)
                                              : reinterpret_cast<const float4*>(dbase + t.atoms);
    return dpx::launch_fill_f64(s, atoms, reinterpret_cast<const int*>(dbase + t.off), d.n_ions,
                                reinterpret_cast<const double*>(dbase + t.aff), G,
                                reinterpret_cast<const int64_t*>(dbase + t.pref), t.items, t.cen, d.scale,
                                t.n_boxes ? reinterpret_cast<const float4*>(dbase + t.boxes) : nullptr,
                                (int)t.n_boxes, reinterpret_cast<double4_32a*>(grid));
}

}  // namespace dpxh
