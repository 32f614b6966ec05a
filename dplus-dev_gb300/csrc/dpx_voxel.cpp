// dpx_voxel.cpp — voxelized solvent of a PDB leaf: the excluded-volume and
// solvation-layer boxes that the amplitude fill adds as a second direct sum.
//
// Follows PDBAmplitude::FindPDBRanges (PDBAmplitude.cpp:710-749) and
// CalculateSolventSpace (VoxelizedSolvent.cpp:4-190) with its helpers
// MarkVoxelsNeighboringAtoms (:388-420), Floodfill3D (:422-440),
// MarkLayerOfSolvent (:192-262) and ReduceSolventSpaceToIrregularBoxes
// (:265-386), on the reference's voxel space layout (SolventSpace,
// Amplitude.cpp:4084-4120: x-major, z padded to a multiple of 16).
// Host code: the box construction is a greedy, order-dependent scan.
#include "dpx_host.h"

#include <cmath>
#include <cstring>
#include <algorithm>
#include <array>
#include <queue>
#include <vector>

using namespace dpxh;

namespace {

enum : signed char {
    kBlue = 0,       // unassigned
    kGreen = 1,      // atoms / excluded volume
    kRed = 2,        // probe shell around the atoms
    kLightBlue = 3,  // bulk solvent
    kPink = 4,       // solvation layer
    kYellow = 5,     // excluded volume already in a box
    kGrey = 6,       // solvation already in a box
    kMarker = 8,     // the fixed marker block CalculateSolventSpace writes after the layer
};

struct Space {
    int64_t xs = 0, ys = 0, zs = 0, plane = 0;
    std::vector<signed char> v;
    void allocate(int64_t x, int64_t y, int64_t z) {
        xs = x;
        ys = y;
        zs = z + (15 - (z + 15) % 16);  // pad z to a multiple of 16
        plane = zs * ys;
        v.assign((size_t)(xs * plane), kBlue);
    }
    signed char& at(int64_t x, int64_t y, int64_t z) { return v[(size_t)(x * plane + y * zs + z)]; }
};

struct Box {
    float com[3];
    int dims[3];
};

struct Voxelizer {
    const float* xyz;
    const float* rad;
    int64_t n;
    double step, probe, thick;
    double xMin, xMax, yMin, yMax, zMin, zMax;
    Space S;

    void ranges() {
        const double dist = std::max(probe, thick) + 2.0 * step;
        float x0 = xyz[0] - rad[0], x1 = xyz[0] + rad[0];
        float y0 = xyz[1] - rad[0], y1 = xyz[1] + rad[0];
        float z0 = xyz[2] - rad[0], z1 = xyz[2] + rad[0];
        for (int64_t i = 1; i < n; ++i) {
            const float* p = xyz + 3 * i;
            x0 = std::min(x0, p[0] - rad[i]);
            x1 = std::max(x1, p[0] + rad[i]);
            y0 = std::min(y0, p[1] - rad[i]);
            y1 = std::max(y1, p[1] + rad[i]);
            z0 = std::min(z0, p[2] - rad[i]);
            z1 = std::max(z1, p[2] + rad[i]);
        }
        xMin = (double)x0 - dist;
        xMax = (double)x1 + dist;
        yMin = (double)y0 - dist;
        yMax = (double)y1 + dist;
        zMin = (double)z0 - dist;
        zMax = (double)z1 + dist;
        xMax = xMin + double(int(2.0 + (xMax - xMin) / step)) * step;
        yMax = yMin + double(int(2.0 + (yMax - yMin) / step)) * step;
        zMax = zMin + double(int(2.0 + (zMax - zMin) / step)) * step;
    }

    // voxels within rad + rSol of an atom centre, currently `from`, become `to`
    void mark_near_atoms(double rSol, signed char from, signed char to) {
        for (int64_t i = 0; i < n; ++i) {
            const double px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
            const double dd = (double)rad[i] + rSol;
            const int reach = 2 + int(dd / step);
            const int xc = int((px - xMin) / step), yc = int((py - yMin) / step), zc = int((pz - zMin) / step);
            const int hx = std::min(xc + reach, (int)S.xs), hy = std::min(yc + reach, (int)S.ys),
                      hz = std::min(zc + reach, (int)S.zs);
            for (int h = std::max(0, xc - reach); h < hx; ++h)
                for (int k = std::max(0, yc - reach); k < hy; ++k)
                    for (int l = std::max(0, zc - reach); l < hz; ++l) {
                        signed char& c = S.at(h, k, l);
                        if (c != from) continue;
                        const double dx = xMin + double(h) * step - px, dy = yMin + double(k) * step - py,
                                     dz = zMin + double(l) * step - pz;
                        if (std::sqrt(dx * dx + dy * dy + dz * dz) <= dd) c = to;
                    }
        }
    }

    // 26-connected breadth-first fill from (i, j, k)
    void flood(int i, int j, int k, signed char from, signed char to) {
        if (S.at(i, j, k) != from) return;
        std::queue<std::array<int, 3>> q;
        S.at(i, j, k) = to;
        q.push({i, j, k});
        while (!q.empty()) {
            const auto p = q.front();
            q.pop();
            for (int a = std::max(0, p[0] - 1); a <= std::min((int)S.xs - 1, p[0] + 1); ++a)
                for (int b = std::max(0, p[1] - 1); b <= std::min((int)S.ys - 1, p[1] + 1); ++b)
                    for (int c = std::max(0, p[2] - 1); c <= std::min((int)S.zs - 1, p[2] + 1); ++c) {
                        signed char& v = S.at(a, b, c);
                        if (v != from) continue;
                        v = to;
                        q.push({a, b, c});
                    }
        }
    }

    // voxels of `type` touching a `neighbor` voxel (interior voxels only) stamp a
    // ball of radius round(radius / step): its `fromType` voxels become `toType`
    void mark_layer(double radius, signed char type, signed char neighbor, signed char toType, signed char fromType) {
        const int disc = int(0.5 + radius / step);
        std::vector<std::array<int, 3>> seeds;
        for (int64_t i = 1; i < S.xs - 1; ++i)
            for (int64_t j = 1; j < S.ys - 1; ++j)
                for (int64_t k = 1; k < S.zs - 1; ++k) {
                    if (S.at(i, j, k) != type) continue;
                    bool touch = false;
                    for (int a = -1; a <= 1 && !touch; ++a)
                        for (int b = -1; b <= 1 && !touch; ++b)
                            for (int c = -1; c <= 1 && !touch; ++c) touch = S.at(i + a, j + b, k + c) == neighbor;
                    if (touch) seeds.push_back({(int)i, (int)j, (int)k});
                }
        for (const auto& s : seeds) {
            const int m1 = std::min((int)S.xs - 1, s[0] + disc), n1 = std::min((int)S.ys - 1, s[1] + disc),
                      p1 = std::min((int)S.zs - 1, s[2] + disc);
            for (int m = std::max(0, s[0] - disc); m <= m1; ++m)
                for (int nn = std::max(0, s[1] - disc); nn <= n1; ++nn)
                    for (int p = std::max(0, s[2] - disc); p <= p1; ++p) {
                        signed char& v = S.at(m, nn, p);
                        if (v != fromType) continue;
                        const double d = std::sqrt(double((m - s[0]) * (m - s[0]) + (nn - s[1]) * (nn - s[1]) +
                                                          (p - s[2]) * (p - s[2])));
                        if (d <= disc) v = toType;
                    }
        }
    }

    // greedy boxes over `designation` voxels in x, y, z scan order
    void reduce(signed char designation, signed char used, std::vector<Box>& out) {
        for (int64_t xb = 0; xb < S.xs; ++xb)
            for (int64_t yb = 0; yb < S.ys; ++yb)
                for (int64_t zb = 0; zb < S.zs; ++zb) {
                    if (S.at(xb, yb, zb) != designation) continue;
                    int64_t lx = 0, ly = 0, lz = 0;  // zero-based extents
                    bool dx = false, dy = false, dz = false;
                    while (!(dx && dy && dz)) {
                        if (!dx) {
                            ++lx;
                            bool ok = xb + lx < S.xs;
                            for (int64_t y = yb; ok && y <= yb + ly; ++y)
                                for (int64_t z = zb; ok && z <= zb + lz; ++z) ok = S.at(xb + lx, y, z) == designation;
                            if (!ok) {
                                dx = true;
                                --lx;
                            }
                        }
                        if (!dy) {
                            ++ly;
                            bool ok = yb + ly < S.ys;
                            for (int64_t x = xb; ok && x <= xb + lx; ++x)
                                for (int64_t z = zb; ok && z <= zb + lz; ++z) ok = S.at(x, yb + ly, z) == designation;
                            if (!ok) {
                                dy = true;
                                --ly;
                            }
                        }
                        if (!dz) {
                            ++lz;
                            bool ok = zb + lz < S.zs;
                            for (int64_t x = xb; ok && x <= xb + lx; ++x)
                                for (int64_t y = yb; ok && y <= yb + ly; ++y) ok = S.at(x, y, zb + lz) == designation;
                            if (!ok) {
                                dz = true;
                                --lz;
                            }
                        }
                    }
                    Box b;
                    b.com[0] = float(xMin + (double(xb) + double(lx) / 2.0) * step);
                    b.com[1] = float(yMin + (double(yb) + double(ly) / 2.0) * step);
                    b.com[2] = float(zMin + (double(zb) + double(lz) / 2.0) * step);
                    b.dims[0] = (int)lx + 1;
                    b.dims[1] = (int)ly + 1;
                    b.dims[2] = (int)lz + 1;
                    out.push_back(b);
                    for (int64_t x = xb; x <= xb + lx; ++x)
                        for (int64_t y = yb; y <= yb + ly; ++y)
                            for (int64_t z = zb; z <= zb + lz; ++z) S.at(x, y, z) = used;
                }
    }

    void run(bool fill_holes, std::vector<Box>& excluded, std::vector<Box>& layer) {
        ranges();
        S.allocate(int64_t((xMax - xMin) / step), int64_t((yMax - yMin) / step), int64_t((zMax - zMin) / step));
        mark_near_atoms(0.0, kBlue, kGreen);
        if (probe > 0.) mark_near_atoms(probe, kBlue, kRed);
        if (fill_holes) {
            flood(0, 0, 0, kBlue, kLightBlue);
            for (auto& c : S.v)
                if (c == kBlue) c = kGreen;  // enclosed cavities count as excluded volume
        } else {
            for (auto& c : S.v)
                if (c == kBlue) c = kLightBlue;
        }
        if (probe > 0.) {
            mark_layer(probe, kLightBlue, kRed, kPink, kRed);
            if (probe < thick)
                mark_layer(std::fabs(thick - probe), kPink, kLightBlue, kPink, kLightBlue);
            else
                mark_layer(std::fabs(thick - probe), kPink, kLightBlue, kLightBlue, kPink);
            mark_near_atoms(0.0, kPink, -1);  // no solvation inside an atom
            for (auto& c : S.v)
                if (c == kRed) c = kGreen;
            // the fixed block of CalculateSolventSpace (VoxelizedSolvent.cpp:77-88):
            // per x slice, y in [1, 1/step], z in [1, 4], written on the flat array
            const int per_nm = int(1. / step);
            const int64_t total = (int64_t)S.v.size();
            for (int64_t x = 0; x < S.xs; ++x)
                for (int i = 0; i < per_nm; ++i)
                    for (int z = 1; z <= 4; ++z) {
                        const int64_t at = x * S.plane + int64_t(1 + i) * S.zs + z;
                        if (at < total) S.v[(size_t)at] = kMarker;
                    }
        }
        reduce(kGreen, kYellow, excluded);
        reduce(kPink, kGrey, layer);
    }
};

}  // namespace

struct dpx_boxes_s {
    std::vector<Box> sets[2];  // 0 excluded volume, 1 solvation layer
    double step;
    int64_t dims[3];
};

extern "C" {

int dpx_voxel_solvent(int64_t n_atoms, const float* xyz, const float* radii, double voxel_step, double probe_radius,
                      double solvation_thickness, int fill_holes, dpx_boxes* out) {
    if (!out || n_atoms <= 0 || !xyz || !radii) return fail(DPX_ERR_ARG, "no atoms");
    if (!(voxel_step > 0)) return fail(DPX_ERR_ARG, "voxel_step must be positive");
    *out = nullptr;
    Voxelizer V{xyz, radii, n_atoms, voxel_step, probe_radius, solvation_thickness, 0, 0, 0, 0, 0, 0, {}};
    V.ranges();
    const double cells = ((V.xMax - V.xMin) / voxel_step + 1) * ((V.yMax - V.yMin) / voxel_step + 1) *
                         ((V.zMax - V.zMin) / voxel_step + 16);
    if (cells > 4.0e9) return fail(DPX_ERR_ARG, "voxel space of %.3g voxels is too large", cells);
    auto* b = new dpx_boxes_s;
    b->step = voxel_step;
    V.run(fill_holes != 0, b->sets[0], b->sets[1]);
    b->dims[0] = V.S.xs;
    b->dims[1] = V.S.ys;
    b->dims[2] = V.S.zs;
    *out = b;
    return DPX_OK;
}

int64_t dpx_boxes_count(dpx_boxes b, int which) {
    if (!b || which < 0 || which > 1) return -1;
    return (int64_t)b->sets[which].size();
}

int dpx_boxes_get(dpx_boxes b, int which, float* com, int* dims) {
    if (!b || which < 0 || which > 1) return fail(DPX_ERR_ARG, "bad box set");
    const auto& s = b->sets[which];
    for (size_t i = 0; i < s.size(); ++i) {
        if (com) std::memcpy(com + 3 * i, s[i].com, 3 * sizeof(float));
        if (dims) std::memcpy(dims + 3 * i, s[i].dims, 3 * sizeof(int));
    }
    return DPX_OK;
}

int dpx_boxes_space(dpx_boxes b, int64_t* dims) {
    if (!b || !dims) return fail(DPX_ERR_ARG, "NULL argument");
    for (int k = 0; k < 3; ++k) dims[k] = b->dims[k];
    return DPX_OK;
}

int dpx_boxes_free(dpx_boxes b) {
    delete b;
    return DPX_OK;
}

}  // extern "C"
