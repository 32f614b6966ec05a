// dpx_fill.cu — amplitude grid fill of PDB leaves on the JacobianSphereGrid,
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
// column chunks of CPT cells; a job's item_pref[i] is the first item after
// shell i.  The FP32 fill is one persistent launch over a batch of jobs
// (structures of any size, on grids of any size): blocks take tiles of THREADS
// items of one job from an atomic counter until the batch is done.
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
// fill_tile computes THREADS consecutive work items of one job; the job's
// fields arrive as scalar __restrict__ arguments so that the inner loop keeps
// them in registers.
// --------------------------------------------------------------------------
// Voxelized-solvent boxes (PDBAmplitude.cpp:277-314): each adds
//   w prod_a [L_a sinc(q_a L_a / 2)] e^{i q.c}
// with the same row factoring as the atoms: the z factor and e^{+-i q_z c_z}
// are shared by the row, the mirror cell differs only in the sign of q_z.
// Boxes arrive sorted by extent, so the per-column x * y factor and the z
// factor are recomputed only when an extent changes (as the reference kernel
// caches its x factor, PDBAmplitudeCUDA.cu:50-58); each box then costs one
// sincos per row and one per column.  Boxes are staged THREADS / 2 at a time
// (two float4 each) in the atom tile.
// sin(h)/h.  The SFU sine has an absolute error near 1e-7-1e-6, which is a
// large RELATIVE error of sin(h)/h for small h (low q, where every box adds in
// phase): below |h| = 0.5 the Taylor series 1 - h^2/6 + h^4/120 - h^6/5040
// (truncation < 1.1e-8) is used instead.
__device__ __forceinline__ float sinc_f(float h) {
    const float h2 = h * h;
    if (h2 < 0.25f) return fmaf(h2, fmaf(h2, fmaf(h2, -1.f / 5040.f, 1.f / 120.f), -1.f / 6.f), 1.f);
    return __fdividef(__sinf(h), h);
}

// sin and cos of x on the FMA pipe, for the columns that the SFU does not
// take (the SFU is the fill's bound; moving a few of the CPT sincos per item to
// the FMA pipe, which the SFU path leaves half idle, balances the two).  x is
// reduced by pi: n = round(x / pi) by the 1.5 * 2^23 shift, pi in two parts
// (Cody and Waite), y in [-pi/2, pi/2]; sin y = y + y^3 P(y^2) and
// cos y = 1 + y^2 Q(y^2) with P, Q of degree 3, coefficients fitted for this
// kernel by error-weighted least squares on Chebyshev nodes (FP32 evaluation:
// |error| <= 1.1e-7 for sin, 1.6e-7 for cos, against 2^-21.4 for the SFU);
// then both carry (-1)^n, the low bit of the shifted n.
__device__ __forceinline__ void sincos_fma(float x, float* s, float* c) {
    const float nm = fmaf(x, 0.318309886183790672f, 12582912.f);
    const float n = nm - 12582912.f;
    float y = fmaf(-n, 3.140625f, x);
    y = fmaf(-n, 9.67653589793116e-4f, y);
    const float y2 = y * y;
    float ps = fmaf(y2, 2.6000548e-06f, -1.98066147e-04f);
    ps = fmaf(y2, ps, 8.33301712e-03f);
    ps = fmaf(y2, ps, -1.66666567e-01f);
    const float sv = fmaf(y * y2, ps, y);
    float pc = fmaf(y2, 2.31943905e-05f, -1.38559274e-03f);
    pc = fmaf(y2, pc, 4.16639894e-02f);
    pc = fmaf(y2, pc, -4.99999315e-01f);
    const float cv = fmaf(y2, pc, 1.0f);
    const unsigned flip = __float_as_uint(nm) << 31;
    *s = __uint_as_float(__float_as_uint(sv) ^ flip);
    *c = __uint_as_float(__float_as_uint(cv) ^ flip);
}

// sincos of column k: the first KP columns on the FMA pipe, the rest on the SFU.
template <int KP>
__device__ __forceinline__ void column_sincos(int k, float x, float* s, float* c) {
    if (k < KP) sincos_fma(x, s, c);
    else __sincosf(x, s, c);
}

template <int CPT, int THREADS, int KP>
__device__ __forceinline__ void box_sum_f32(const float4* __restrict__ boxes, int n_boxes, const float (&qx)[CPT],
                                            const float (&qy)[CPT], float qz, float (&cc)[CPT], float (&ss)[CPT],
                                            float (&sc)[CPT], float (&cs)[CPT], float4* __restrict__ s_box) {
    float fxy[CPT], fz = 0.f;
    float lx = -1.f, ly = -1.f, lz = -1.f;
    for (int b0 = 0; b0 < n_boxes; b0 += THREADS / 2) {
        const int nb = min(THREADS / 2, n_boxes - b0);
        __syncthreads();
        if (threadIdx.x < 2 * nb) s_box[threadIdx.x] = boxes[2 * (int64_t)b0 + threadIdx.x];
        __syncthreads();
        // per-tile partial sums: near q = 0 every box adds in phase, and adding
        // each small term straight to the running sum would round 1e5 times
        float tcc[CPT], tss[CPT], tsc[CPT], tcs[CPT];
#pragma unroll
        for (int k = 0; k < CPT; ++k) tcc[k] = tss[k] = tsc[k] = tcs[k] = 0.f;
        for (int j = 0; j < nb; ++j) {
            const float4 c = s_box[2 * j], L = s_box[2 * j + 1];
            if (L.x != lx || L.y != ly) {
                lx = L.x;
                ly = L.y;
#pragma unroll
                for (int k = 0; k < CPT; ++k)
                    fxy[k] = L.x * sinc_f(0.5f * qx[k] * L.x) * L.y * sinc_f(0.5f * qy[k] * L.y);
            }
            if (L.z != lz) {
                lz = L.z;
                fz = L.z * sinc_f(0.5f * qz * L.z);
            }
            float sz, cz;
            __sincosf(qz * c.z, &sz, &cz);
            const float wz = c.w * fz, wcz = wz * cz, wsz = wz * sz;
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                float sn, cn;
                column_sincos<KP>(k, fmaf(qy[k], c.y, qx[k] * c.x), &sn, &cn);
                const float tc = fxy[k] * cn, ts = fxy[k] * sn;
                tcc[k] = fmaf(tc, wcz, tcc[k]);
                tss[k] = fmaf(ts, wsz, tss[k]);
                tsc[k] = fmaf(ts, wcz, tsc[k]);
                tcs[k] = fmaf(tc, wsz, tcs[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            cc[k] += tcc[k];
            ss[k] += tss[k];
            sc[k] += tsc[k];
            cs[k] += tcs[k];
        }
    }
}

template <int CPT, int THREADS, bool BOXES, int KP>
__device__ __forceinline__ void fill_tile(const float4* __restrict__ atoms, const int* __restrict__ ion_off, int U,
                                          const float* __restrict__ aff, const int64_t* __restrict__ pref,
                                          const float4* __restrict__ boxes, int n_boxes, float4* __restrict__ grid,
                                          int64_t n_items, int Lp, double step, double cx, double cy, double cz,
                                          int use_center, float scale, double origin, int64_t w,
                                          float4* __restrict__ s_atoms) {
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

    // Four product sums per column instead of two complex accumulators:
    //   cc = sum f c cz, ss = sum f s sz, sc = sum f s cz, cs = sum f c sz
    // with (c, s) = e^{i Pxy}, (cz, sz) = e^{i Pz}; then
    //   F = (cc - ss) + i (sc + cs),  G = (cc + ss) + i (sc - cs),
    // four FMAs per atom and column where the complex products take eight.
    float cc[CPT], ss[CPT], sc[CPT], cs[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) cc[k] = ss[k] = sc[k] = cs[k] = 0.f;

    for (int u = 0; u < U; ++u) {
        const int a0 = ion_off[u], a1 = ion_off[u + 1];
        const float f = aff[(int64_t)u * (Lp + 1) + i];
        for (int t0 = a0; t0 < a1; t0 += THREADS) {
            const int n = min(THREADS, a1 - t0);
            __syncthreads();
            if (threadIdx.x < n) s_atoms[threadIdx.x] = atoms[t0 + threadIdx.x];
            __syncthreads();
            float tcc[CPT], tss[CPT], tsc[CPT], tcs[CPT];
#pragma unroll
            for (int k = 0; k < CPT; ++k) tcc[k] = tss[k] = tsc[k] = tcs[k] = 0.f;
#pragma unroll 2
            for (int j = 0; j < n; ++j) {
                const float4 a = s_atoms[j];
                float sz, cz;
                __sincosf(qz * a.z, &sz, &cz);
#pragma unroll
                for (int k = 0; k < CPT; ++k) {
                    float sn, cn;
                    column_sincos<KP>(k, fmaf(qy[k], a.y, qx[k] * a.x), &sn, &cn);
                    tcc[k] = fmaf(cn, cz, tcc[k]);
                    tss[k] = fmaf(sn, sz, tss[k]);
                    tsc[k] = fmaf(sn, cz, tsc[k]);
                    tcs[k] = fmaf(cn, sz, tcs[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                cc[k] = fmaf(f, tcc[k], cc[k]);
                ss[k] = fmaf(f, tss[k], ss[k]);
                sc[k] = fmaf(f, tsc[k], sc[k]);
                cs[k] = fmaf(f, tcs[k], cs[k]);
            }
        }
    }
    if (BOXES && n_boxes > 0) box_sum_f32<CPT, THREADS, KP>(boxes, n_boxes, qx, qy, qz, cc, ss, sc, cs, s_atoms);
    if (!active) return;

    float fR[CPT], fI[CPT], gR[CPT], gI[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        fR[k] = cc[k] - ss[k];
        fI[k] = sc[k] + cs[k];
        gR[k] = cc[k] + ss[k];
        gI[k] = sc[k] - cs[k];
    }

    float2* g2 = reinterpret_cast<float2*>(grid);
    if (i == 0) {  // origin: every phase is zero; the host's FP64 sum avoids 1e5 in-phase roundings
        g2[0] = make_float2((float)origin, 0.f);
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

__device__ __forceinline__ int job_of_tile(const FillJob* __restrict__ jobs, int n_jobs, int64_t tile) {
    int lo = 0, hi = n_jobs - 1;  // last job with tile_start <= tile
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].tile_start <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int CPT, int THREADS, bool BOXES, int KP>
__device__ __forceinline__ void run_tile(const FillJob& J, int64_t tile, float4* s_atoms) {
    fill_tile<CPT, THREADS, BOXES, KP>(J.atoms, J.ion_off, J.U, J.aff_f32, J.pref, J.boxes, J.n_boxes, J.grid, J.n_items, J.Lp,
                            J.step, J.cx, J.cy, J.cz, J.use_center, J.scale, J.origin,
                            (tile - J.tile_start) * THREADS + threadIdx.x, s_atoms);
}

// Persistent form: one CTA per resident slot, tiles of every job pulled from
// an atomic counter; the job record is staged once per tile in shared memory.
template <int CPT, int THREADS, int KP>
__global__ void __launch_bounds__(THREADS) fill_f32_persistent(const FillJob* __restrict__ jobs, int n_jobs,
                                                               int64_t total_tiles,
                                                               unsigned long long* __restrict__ counter) {
    __shared__ float4 s_atoms[THREADS];
    __shared__ FillJob s_job;
    __shared__ long long s_tile;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const long long t = (long long)atomicAdd(counter, 1ull);
            s_tile = t;
            if (t < total_tiles) s_job = jobs[job_of_tile(jobs, n_jobs, t)];
        }
        __syncthreads();
        const int64_t tile = s_tile;
        if (tile >= total_tiles) break;
        const FillJob J = s_job;
        run_tile<CPT, THREADS, false, KP>(J, tile, s_atoms);
    }
}

// Flat form: one CTA per tile over the whole batch; the hardware block
// scheduler hands out the tiles in order.  BOXES compiles the voxelized-solvent
// sum in (a batch with boxes runs this form; without, the leaner code keeps
// the atom loop's registers free).
template <int CPT, int THREADS, bool BOXES, int KP>
__global__ void __launch_bounds__(THREADS, 512 / THREADS) fill_f32_flat(const FillJob* __restrict__ jobs, int n_jobs) {
    __shared__ float4 s_atoms[THREADS];
    const int64_t tile = blockIdx.x;
    const FillJob J = jobs[job_of_tile(jobs, n_jobs, tile)];
    run_tile<CPT, THREADS, BOXES, KP>(J, tile, s_atoms);
}

// --------------------------------------------------------------------------
// Plain FP64: FP64 q vector (sincospi), FP64 phases, FP64 sincos, FP64 sums.
// One job per launch.
// --------------------------------------------------------------------------
template <int CPT, int THREADS>
__global__ void __launch_bounds__(THREADS) fill_f64_kernel(const float4* __restrict__ atoms,
                                                           const int* __restrict__ ion_off, int U,
                                                           const double* __restrict__ aff, int Lp, double step,
                                                           const int64_t* __restrict__ pref, double cx, double cy,
                                                           double cz, double scale, const float4* __restrict__ boxes,
                                                           int n_boxes, double4_32a* __restrict__ grid) {
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

    // the four product sums of the FP32 fill, in FP64
    double cc[CPT], ss[CPT], sc[CPT], cs[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) cc[k] = ss[k] = sc[k] = cs[k] = 0.0;

    for (int u = 0; u < U; ++u) {
        const int a0 = ion_off[u], a1 = ion_off[u + 1];
        double tcc[CPT], tss[CPT], tsc[CPT], tcs[CPT];
#pragma unroll
        for (int k = 0; k < CPT; ++k) tcc[k] = tss[k] = tsc[k] = tcs[k] = 0.0;
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
                    double sn, cn;
                    sincos(qx[k] * a.x + qy[k] * a.y, &sn, &cn);
                    tcc[k] = fma(cn, cz, tcc[k]);
                    tss[k] = fma(sn, sz, tss[k]);
                    tsc[k] = fma(sn, cz, tsc[k]);
                    tcs[k] = fma(cn, sz, tcs[k]);
                }
            }
        }
        const double f = aff[(int64_t)u * (Lp + 1) + i];
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            cc[k] = fma(f, tcc[k], cc[k]);
            ss[k] = fma(f, tss[k], ss[k]);
            sc[k] = fma(f, tsc[k], sc[k]);
            cs[k] = fma(f, tcs[k], cs[k]);
        }
    }
    // voxelized-solvent boxes in FP64 (box data are the reference's floats),
    // the x * y and z extent factors cached across boxes sorted by extent
    double fxy[CPT], fz = 0.0, lx = -1.0, ly = -1.0, lz = -1.0;
    for (int b0 = 0; b0 < n_boxes; b0 += THREADS / 2) {
        const int nb = min(THREADS / 2, n_boxes - b0);
        __syncthreads();
        if (threadIdx.x < 2 * nb) {
            const float4 v = boxes[2 * (int64_t)b0 + threadIdx.x];
            s_atoms[threadIdx.x] = make_double4_32a(v.x, v.y, v.z, v.w);
        }
        __syncthreads();
        for (int j = 0; j < nb; ++j) {
            const double4_32a c = s_atoms[2 * j], L = s_atoms[2 * j + 1];
            if (L.x != lx || L.y != ly) {
                lx = L.x;
                ly = L.y;
#pragma unroll
                for (int k = 0; k < CPT; ++k) {
                    const double hx = 0.5 * qx[k] * L.x, hy = 0.5 * qy[k] * L.y;
                    fxy[k] = L.x * (hx == 0.0 ? 1.0 : sin(hx) / hx) * L.y * (hy == 0.0 ? 1.0 : sin(hy) / hy);
                }
            }
            if (L.z != lz) {
                lz = L.z;
                const double h = 0.5 * qz * L.z;
                fz = L.z * (h == 0.0 ? 1.0 : sin(h) / h);
            }
            double sz, cz;
            sincos(qz * c.z, &sz, &cz);
            const double wz = c.w * fz, wcz = wz * cz, wsz = wz * sz;
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                double sn, cn;
                sincos(qx[k] * c.x + qy[k] * c.y, &sn, &cn);
                const double tc = fxy[k] * cn, ts = fxy[k] * sn;
                cc[k] = fma(tc, wcz, cc[k]);
                ss[k] = fma(ts, wsz, ss[k]);
                sc[k] = fma(ts, wcz, sc[k]);
                cs[k] = fma(tc, wsz, cs[k]);
            }
        }
    }
    double fR[CPT], fI[CPT], gR[CPT], gI[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        fR[k] = cc[k] - ss[k];
        fI[k] = sc[k] + cs[k];
        gR[k] = cc[k] + ss[k];
        gI[k] = sc[k] - cs[k];
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

template <int CPT, int TH, int KP>
cudaError_t launch_batch(cudaStream_t s, const FillJob* d_jobs, int n_jobs, int64_t total_tiles,
                         unsigned long long* d_counter, bool persistent, bool boxes) {
    if (!persistent || boxes) {
        if (total_tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
        if (boxes) fill_f32_flat<CPT, TH, true, KP><<<(unsigned)total_tiles, TH, 0, s>>>(d_jobs, n_jobs);
        else fill_f32_flat<CPT, TH, false, KP><<<(unsigned)total_tiles, TH, 0, s>>>(d_jobs, n_jobs);
        return cudaGetLastError();
    }
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fill_f32_persistent<CPT, TH, KP>, TH, 0);
    if (e != cudaSuccess) return e;
    int64_t blocks = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
    if (blocks > total_tiles) blocks = total_tiles;
    e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    fill_f32_persistent<CPT, TH, KP><<<(unsigned)blocks, TH, 0, s>>>(d_jobs, n_jobs, total_tiles, d_counter);
    return cudaGetLastError();
}

}  // namespace

int64_t fill_items(const Geom& g, int cpt, int64_t* pref) {
    pref[0] = 1;
    for (int i = 1; i <= g.Lp; ++i) pref[i] = pref[i - 1] + (int64_t)(3 * i / 2 + 1) * ((3 * i + cpt - 1) / cpt);
    return pref[g.Lp];
}

cudaError_t launch_fill_f32_batch(cudaStream_t s, const FillJob* d_jobs, int n_jobs, int64_t total_tiles,
                                  unsigned long long* d_counter, int cells_per_thread, int block, int poly,
                                  bool persistent, bool boxes) {
    if (n_jobs <= 0 || total_tiles <= 0) return cudaSuccess;
#define DPX_FILL_CASE(CPT, TH, KP)                                    \
    if (cells_per_thread == CPT && block == TH && poly == KP)         \
        return launch_batch<CPT, TH, KP>(s, d_jobs, n_jobs, total_tiles, d_counter, persistent, boxes);
    DPX_FILL_CASE(2, 256, 0) DPX_FILL_CASE(4, 128, 0) DPX_FILL_CASE(4, 256, 0) DPX_FILL_CASE(6, 128, 0)
    DPX_FILL_CASE(6, 256, 0) DPX_FILL_CASE(8, 128, 0) DPX_FILL_CASE(8, 256, 0)
    DPX_FILL_CASE(8, 128, 1) DPX_FILL_CASE(8, 128, 2) DPX_FILL_CASE(8, 128, 3)
#undef DPX_FILL_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_fill_f64(cudaStream_t s, const float4* atoms, const int* ion_off, int U, const double* aff,
                            const Geom& g, const int64_t* d_pref, int64_t n_items, const double center[3],
                            double scale, const float4* boxes, int n_boxes, double4_32a* grid) {
    if (n_items <= 0) return cudaSuccess;
    fill_f64_kernel<kFill64Cells, 128><<<blocks_for(n_items, 128), 128, 0, s>>>(
        atoms, ion_off, U, aff, g.Lp, g.step, d_pref, center[0], center[1], center[2], scale, boxes, n_boxes, grid);
    return cudaGetLastError();
}

}  // namespace dpx
