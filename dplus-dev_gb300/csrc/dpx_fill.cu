// dpx_fill.cu — amplitude grid fill of a PDB leaf on the JacobianSphereGrid,
//   F(q) = scale * sum_u aff_u(|q|) sum_{j in u} e^{i q.r_j}
// (D+ PDBAmplitude.cpp:243-317 evaluated on every cell by Grid.cpp:760-826;
// the reference GPU kernel is PDBAmplitudeCUDA.cu:134-186).
//
// Symmetry used to cut the sin/cos work (exact identities, real form factors):
//  * within theta row t of shell i all cells share q_z = q_i cos(theta_t); the
//    phase splits as P_xy + P_z with P_z = q_z z.  One sincos of P_z per atom
//    serves the whole row, and one sincos of P_xy gives both
//        F(t, p)      = sum f e^{i(P_xy + P_z)}
//        G(t, p)      = sum f e^{i(P_xy - P_z)}  = F at the z-mirror (3i - t, p);
//  * Friedel: F(-q) = conj F(q), and the antipode of (t, p) is (3i - t, p + 3i).
// So a work item covers rows t <= 3i/2 and columns p < 3i and writes four
// cells: (t, p) = F, (t, p+3i) = conj G, (3i-t, p+3i) = conj F, (3i-t, p) = G
// (on the equator row, 3i even and t = 3i/2, G = F and only two are written).
// Sin/cos evaluations per cell drop from 1 to (1 + 1/CPT) / 4.
//
// Work items: origin first, then per shell (floor(3i/2)+1) rows x ceil(3i/CPT)
// column chunks of CPT cells; item_pref[i] is the first item after shell i.
#include "dpx_internal.h"

#include <cuda_runtime.h>
#include <cstdint>

namespace dpx {

namespace {

struct Item {
    int i, t, p0;  // shell, theta row, first phi column
};

__device__ __forceinline__ Item find_item(int64_t w, const int64_t* __restrict__ pref, int Lp, int cpt) {
    // smallest shell i in [1, Lp] with pref[i] > w (pref[0] = 1 covers the origin)
    int lo = 1, hi = Lp;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (pref[mid] > w) hi = mid;
        else lo = mid + 1;
    }
    const int i = lo;
    const int64_t local = w - pref[i - 1];
    const int nch = (3 * i + cpt - 1) / cpt;
    Item it;
    it.i = i;
    it.t = (int)(local / nch);
    it.p0 = (int)(local - (int64_t)it.t * nch) * cpt;
    return it;
}

template <typename V2>
__device__ __forceinline__ void store_quad(V2* __restrict__ g2, int i, int t, int p, V2 F, V2 G) {
    // g2 points at the {re, im} half of each cell (stride 2 of V2)
    const int64_t b = shell_base(i), n = 6 * (int64_t)i, h = 3 * (int64_t)i;
    const int64_t c1 = b + t * n + p;
    const int64_t c4 = b + (h - t) * n + p;
    V2 cF = F, cG = G;
    cF.y = -F.y;
    cG.y = -G.y;
    g2[2 * c1] = F;
    g2[2 * (c1 + h)] = cG;
    if (2 * t != (int)h) {
        g2[2 * (c4 + h)] = cF;
        g2[2 * c4] = G;
    }
}

// --------------------------------------------------------------------------
// FP32 bulk: FP32 phases, SFU __sincosf, FP32 sums (per atom tile, then scaled
// by the ion's form factor into the cell accumulators); the centring
// translation c is restored per cell as e^{i q.c} in FP64.
// --------------------------------------------------------------------------
template <int CPT, int THREADS>
__global__ void __launch_bounds__(THREADS) fill_f32_kernel(const float4* __restrict__ atoms,
                                                           const int* __restrict__ ion_off, int U,
                                                           const float* __restrict__ aff, int Lp, double step,
                                                           const int64_t* __restrict__ pref, double cx, double cy,
                                                           double cz, int use_center, float scale,
                                                           float4* __restrict__ grid) {
    __shared__ float4 s_atoms[THREADS];
    const int64_t w = (int64_t)blockIdx.x * THREADS + threadIdx.x;
    const int64_t n_items = pref[Lp];
    const bool active = w < n_items;
    Item it{0, 0, 0};
    if (active && w > 0) it = find_item(w, pref, Lp, CPT);
    const int i = it.i;

    float qx[CPT], qy[CPT], qz = 0.f;
    if (i > 0) {
        const float qI = (float)((double)i * step);
        float st, ct;
        sincospif((float)it.t / (float)(3 * i), &st, &ct);
        qz = qI * ct;
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            float sp, cp;
            sincospif((float)(it.p0 + k) / (float)(3 * i), &sp, &cp);
            qx[k] = qI * st * cp;
            qy[k] = qI * st * sp;
        }
    } else {
#pragma unroll
        for (int k = 0; k < CPT; ++k) qx[k] = qy[k] = 0.f;
    }
    const int layer = i;

    float fR[CPT], fI[CPT], gR[CPT], gI[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) fR[k] = fI[k] = gR[k] = gI[k] = 0.f;

    for (int u = 0; u < U; ++u) {
        const int a0 = ion_off[u], a1 = ion_off[u + 1];
        const float f = aff[(int64_t)u * (Lp + 1) + layer];
        for (int t0 = a0; t0 < a1; t0 += THREADS) {
            const int n = min(THREADS, a1 - t0);
            __syncthreads();
            if (threadIdx.x < n) s_atoms[threadIdx.x] = atoms[t0 + threadIdx.x];
            __syncthreads();
            float tFr[CPT], tFi[CPT], tGr[CPT], tGi[CPT];
#pragma unroll
            for (int k = 0; k < CPT; ++k) tFr[k] = tFi[k] = tGr[k] = tGi[k] = 0.f;
#pragma unroll 2
            for (int j = 0; j < n; ++j) {
                const float4 a = s_atoms[j];
                float sz, cz;
                __sincosf(qz * a.z, &sz, &cz);
#pragma unroll
                for (int k = 0; k < CPT; ++k) {
                    float s, c;
                    __sincosf(fmaf(qy[k], a.y, qx[k] * a.x), &s, &c);
                    // e^{i Pxy} e^{+-i Pz}
                    tFr[k] = fmaf(-s, sz, fmaf(c, cz, tFr[k]));
                    tFi[k] = fmaf(c, sz, fmaf(s, cz, tFi[k]));
                    tGr[k] = fmaf(s, sz, fmaf(c, cz, tGr[k]));
                    tGi[k] = fmaf(-c, sz, fmaf(s, cz, tGi[k]));
                }
            }
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                fR[k] = fmaf(f, tFr[k], fR[k]);
                fI[k] = fmaf(f, tFi[k], fI[k]);
                gR[k] = fmaf(f, tGr[k], gR[k]);
                gI[k] = fmaf(f, tGi[k], gI[k]);
            }
        }
    }
    if (!active) return;

    float2* g2 = reinterpret_cast<float2*>(grid);
    if (i == 0) {  // origin: every phase is zero
        g2[0] = make_float2(fR[0] * scale, fI[0] * scale);
        return;
    }
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const int p = it.p0 + k;
        if (p >= 3 * i) break;
        float2 F = make_float2(fR[k] * scale, fI[k] * scale);
        float2 G = make_float2(gR[k] * scale, gI[k] * scale);
        if (use_center) {
            const double pxy = (double)qx[k] * cx + (double)qy[k] * cy, pz = (double)qz * cz;
            double s1, c1, s2, c2;
            sincos(pxy + pz, &s1, &c1);
            sincos(pxy - pz, &s2, &c2);
            F = make_float2((float)(F.x * c1 - F.y * s1), (float)(F.x * s1 + F.y * c1));
            G = make_float2((float)(G.x * c2 - G.y * s2), (float)(G.x * s2 + G.y * c2));
        }
        store_quad(g2, i, it.t, p, F, G);
    }
}

// --------------------------------------------------------------------------
// Plain FP64: FP64 q vector (sincospi), FP64 phases, FP64 sincos, FP64 sums.
// --------------------------------------------------------------------------
template <int CPT, int THREADS>
__global__ void __launch_bounds__(THREADS) fill_f64_kernel(const float4* __restrict__ atoms,
                                                           const int* __restrict__ ion_off, int U,
                                                           const double* __restrict__ aff, int Lp, double step,
                                                           const int64_t* __restrict__ pref, double cx, double cy,
                                                           double cz, double scale, double4_32a* __restrict__ grid) {
    __shared__ double4_32a s_atoms[THREADS];
    const int64_t w = (int64_t)blockIdx.x * THREADS + threadIdx.x;
    const int64_t n_items = pref[Lp];
    const bool active = w < n_items;
    Item it{0, 0, 0};
    if (active && w > 0) it = find_item(w, pref, Lp, CPT);
    const int i = it.i;

    double qx[CPT], qy[CPT], qz = 0.0;
    if (i > 0) {
        const double qI = (double)i * step;
        double st, ct;
        sincospi((double)it.t / (double)(3 * i), &st, &ct);
        qz = qI * ct;
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            double sp, cp;
            sincospi((double)(it.p0 + k) / (double)(3 * i), &sp, &cp);
            qx[k] = qI * st * cp;
            qy[k] = qI * st * sp;
        }
    } else {
#pragma unroll
        for (int k = 0; k < CPT; ++k) qx[k] = qy[k] = 0.0;
    }

    double fR[CPT], fI[CPT], gR[CPT], gI[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) fR[k] = fI[k] = gR[k] = gI[k] = 0.0;

    for (int u = 0; u < U; ++u) {
        const int a0 = ion_off[u], a1 = ion_off[u + 1];
        double sFr[CPT], sFi[CPT], sGr[CPT], sGi[CPT];
#pragma unroll
        for (int k = 0; k < CPT; ++k) sFr[k] = sFi[k] = sGr[k] = sGi[k] = 0.0;
        for (int t0 = a0; t0 < a1; t0 += THREADS) {
            const int n = min(THREADS, a1 - t0);
            __syncthreads();
            if (threadIdx.x < n) {
                const float4 a = atoms[t0 + threadIdx.x];
                s_atoms[threadIdx.x] = make_double4_32a(a.x, a.y, a.z, 0.0);
            }
            __syncthreads();
            for (int j = 0; j < n; ++j) {
                const double4_32a a = s_atoms[j];
                double sz, cz;
                sincos(qz * a.z, &sz, &cz);
#pragma unroll
                for (int k = 0; k < CPT; ++k) {
                    double s, c;
                    sincos(qx[k] * a.x + qy[k] * a.y, &s, &c);
                    sFr[k] += c * cz - s * sz;
                    sFi[k] += s * cz + c * sz;
                    sGr[k] += c * cz + s * sz;
                    sGi[k] += s * cz - c * sz;
                }
            }
        }
        const double f = aff[(int64_t)u * (Lp + 1) + i];
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            fR[k] += f * sFr[k];
            fI[k] += f * sFi[k];
            gR[k] += f * sGr[k];
            gI[k] += f * sGi[k];
        }
    }
    if (!active) return;

    double2* g2 = reinterpret_cast<double2*>(grid);
    if (i == 0) {
        g2[0] = make_double2(fR[0] * scale, fI[0] * scale);
        return;
    }
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const int p = it.p0 + k;
        if (p >= 3 * i) break;
        double2 F = make_double2(fR[k] * scale, fI[k] * scale);
        double2 G = make_double2(gR[k] * scale, gI[k] * scale);
        if (cx != 0.0 || cy != 0.0 || cz != 0.0) {
            const double pxy = qx[k] * cx + qy[k] * cy, pz = qz * cz;
            double s1, c1, s2, c2;
            sincos(pxy + pz, &s1, &c1);
            sincos(pxy - pz, &s2, &c2);
            F = make_double2(F.x * c1 - F.y * s1, F.x * s1 + F.y * c1);
            G = make_double2(G.x * c2 - G.y * s2, G.x * s2 + G.y * c2);
        }
        store_quad(g2, i, it.t, p, F, G);
    }
}

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

int64_t fill_items(const Geom& g, int cpt, int64_t* pref) {
    pref[0] = 1;
    for (int i = 1; i <= g.Lp; ++i) pref[i] = pref[i - 1] + (int64_t)(3 * i / 2 + 1) * ((3 * i + cpt - 1) / cpt);
    return pref[g.Lp];
}

cudaError_t launch_fill_f32(cudaStream_t s, const float4* atoms, const int* ion_off, int U, const float* aff,
                            const Geom& g, const int64_t* d_pref, int64_t n_items, const double center[3],
                            float scale, float4* grid, int cells_per_thread, int block) {
    if (n_items <= 0) return cudaSuccess;
    const int use_center = (center[0] != 0.0 || center[1] != 0.0 || center[2] != 0.0);
#define DPX_FILL_CASE(CPT, TH)                                                                                  \
    if (cells_per_thread == CPT && block == TH) {                                                              \
        fill_f32_kernel<CPT, TH><<<blocks_for(n_items, TH), TH, 0, s>>>(atoms, ion_off, U, aff, g.Lp, g.step,  \
                                                                       d_pref, center[0], center[1], center[2], \
                                                                       use_center, scale, grid);               \
        return cudaGetLastError();                                                                             \
    }
    DPX_FILL_CASE(2, 256) DPX_FILL_CASE(4, 128) DPX_FILL_CASE(4, 256) DPX_FILL_CASE(6, 128) DPX_FILL_CASE(6, 256)
    DPX_FILL_CASE(8, 128) DPX_FILL_CASE(8, 256)
#undef DPX_FILL_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_fill_f64(cudaStream_t s, const float4* atoms, const int* ion_off, int U, const double* aff,
                            const Geom& g, const int64_t* d_pref, int64_t n_items, const double center[3],
                            double scale, double4_32a* grid) {
    if (n_items <= 0) return cudaSuccess;
    fill_f64_kernel<kFill64Cells, 128><<<blocks_for(n_items, 128), 128, 0, s>>>(
        atoms, ion_off, U, aff, g.Lp, g.step, d_pref, center[0], center[1], center[2], scale, grid);
    return cudaGetLastError();
}

}  // namespace dpx
