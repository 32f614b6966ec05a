// dpx_harmonic.cu — FP32 amplitude grid by spherical-harmonic (multipole)
// expansion, the same F(q) = scale sum_j f_j(|q|) e^{i q.r_j} (+ voxelized
// solvent) as the direct fill of dpx_fill.cu, evaluated as
//   F(q, theta, phi) = 4 pi sum_l i^l sum_{m>=0} Pbar_lm(cos theta)
//                      [C_lm(q) e^{i m phi} + (m > 0) conj(C_lm(q)) e^{-i m phi}],
//   C_lm(q)          = sum_j f_j(q) j_l(q r_j) Pbar_lm(cos theta_j) e^{-i m phi_j}
// (the plane-wave expansion e^{i q.r} = 4 pi sum_lm i^l j_l(qr) Y*_lm(r^) Y_lm(q^);
// for real f, the m < 0 terms are the conjugates of the m > 0 ones).  Pbar_lm
// are the orthonormal associated Legendre functions (Y_lm = Pbar_lm e^{i m phi}).
// The series is cut at l_i = ceil(x + 3 x^(1/3) + 6), x = q_i R, R the largest
// |r_j| about the centroid: beyond it j_l(x) is below 1e-7 of its peak.
//
// Cost: the direct fill spends one sincos per point and grid cell (divided by
// four through the row and Friedel symmetries); here a point costs
// sum_i (l_i + 1) Bessel values and (l_max + 1)^2 / 2 basis values, the
// analysis is a GEMM-shaped sum (shells x (l, m)) over the points, and the
// synthesis of a theta row costs O(l_i^2 + cells x l_i) independent of the
// number of points.
//
// Kernels (per chunk of points, points being atoms or solvent voxels; a chunk
// is sized so that its basis table stays in L2 while the GEMM re-reads it):
//   hm_basis   Y[k][j] = Pbar_lm(cos theta_j) e^{-i m phi_j}, k = l(l+1)/2 + m
//   hm_bessel  J_l[i][j] = f_j(q_i) j_l(q_i r_j)   (upward recurrence for
//              l <= x, downward continued fraction above)
//   hm_gemm    C[i][k] += sum_j J_l(k)[i][j] Y[k][j]: FP32 products in 64-point
//              sub-tiles, Kahan-compensated across sub-tiles, FP64 across chunks
// then hm_synth writes the grid: per
// theta row t <= 3i/2 the B_m of both exponentials, the 6i cells by a table of
// 6i-th roots of unity, the voxel form factor prod_a s sinc(q_a s / 2) on the
// solvent part (a box of n voxels is exactly the sum of its voxels), the
// centring phase e^{i q.c} in FP64, and the Friedel mirror row.
#include "dpx_internal.h"

#include <cstdint>

namespace dpx {
namespace {

constexpr float kFourPi = 12.566370614359172954f;
constexpr int kGemmShells = 32;  // shells per GEMM block (8 groups of 4)
constexpr int kGemmM = 64;       // m values per GEMM block (2 per lane)
constexpr int kGemmSub = 64;     // points per shared-memory sub-tile

__device__ __forceinline__ int k_of(int l, int m) { return l * (l + 1) / 2 + m; }

// ---------------------------------------------------------------------------
// hm_basis: thread (point j of the chunk, order m); padding points write zeros.
// ab[k] = {a_lm, b_lm} of the recurrence Pbar_lm = a (x Pbar_{l-1,m} - b Pbar_{l-2,m}).
// ---------------------------------------------------------------------------
__global__ void hm_basis(const float4* __restrict__ pts, int64_t n, int64_t chunk_off, int ch, int LM,
                         const float2* __restrict__ ab, float2* __restrict__ Y) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (j >= ch) return;
    const int64_t g = chunk_off + j;
    float ct = 1.f, st = 0.f, ph = 0.f;
    const bool valid = g < n;
    if (valid) {
        const float4 p = pts[g];
        const float rxy = sqrtf(fmaf(p.x, p.x, p.y * p.y));
        const float r = sqrtf(fmaf(p.z, p.z, rxy * rxy));
        if (r > 0.f) {
            ct = p.z / r;
            st = rxy / r;
            ph = atan2f(p.y, p.x);
        }
    }
    float pmm = 0.28209479177387814347f;  // 1 / sqrt(4 pi)
    for (int mm = 1; mm <= m; ++mm) pmm = -sqrtf((2.f * mm + 1.f) / (2.f * mm)) * st * pmm;
    float sm, cm;
    sincosf((float)m * ph, &sm, &cm);  // e^{-i m phi}, accurate argument reduction
    const float er = valid ? cm : 0.f, ei = valid ? -sm : 0.f;
    float p2 = 0.f, p1 = pmm;
    Y[(int64_t)k_of(m, m) * ch + j] = make_float2(p1 * er, p1 * ei);
    for (int l = m + 1; l <= LM; ++l) {
        const float2 c = ab[k_of(l, m)];
        const float p0 = c.x * fmaf(ct, p1, -c.y * p2);
        Y[(int64_t)k_of(l, m) * ch + j] = make_float2(p0 * er, p0 * ei);
        p2 = p1;
        p1 = p0;
    }
}

// ---------------------------------------------------------------------------
// hm_bessel: thread (point j of the chunk, shell i >= 1).  J_l rows are the
// shells i >= imin[l]; J_l starts at joff[l] (in units of ch).
// The weight of a point is its ion's form factor at q_i (atoms: w holds the
// ion index) or its solvent weight in e/nm^3 (voxels).
// ---------------------------------------------------------------------------
constexpr int kMaxL = 192;

template <bool VOXELS>
__global__ void hm_bessel(const float4* __restrict__ pts, int64_t n, int64_t chunk_off, int ch, int Lp, double step,
                          const int* __restrict__ lmax, const int* __restrict__ imin, const int64_t* __restrict__ joff,
                          const float* __restrict__ aff, float* __restrict__ J) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y + 1;
    if (j >= ch) return;
    const int li = lmax[i];
    const int64_t g = chunk_off + j;
    float w = 0.f, r = 0.f;
    if (g < n) {
        const float4 p = pts[g];
        r = sqrtf(fmaf(p.x, p.x, fmaf(p.y, p.y, p.z * p.z)));
        w = VOXELS ? p.w : aff[(int64_t)(int)p.w * (Lp + 1) + i];
    }
    const float x = (float)((double)i * step) * r;
    auto put = [&](int l, float v) { J[(joff[l] + (int64_t)(i - imin[l])) * ch + j] = w * v; };
    if (w == 0.f) {
        for (int l = 0; l <= li; ++l) put(l, 0.f);
        return;
    }
    if (x < 1e-3f) {  // j_0 = 1 - x^2/6, j_1 = x/3, higher orders below 1e-10
        put(0, 1.f - x * x / 6.f);
        if (li >= 1) put(1, x / 3.f);
        for (int l = 2; l <= li; ++l) put(l, 0.f);
        return;
    }
    float s, c;
    sincosf(x, &s, &c);
    const float ix = 1.f / x;
    const float j0 = s * ix;
    // l <= L0 = floor(x): upward recurrence, stable below the turning point
    const int L0 = min((int)x, li);
    put(0, j0);
    float jm = j0, jc = 0.f;
    if (L0 >= 1) {
        jc = (j0 - c) * ix;  // j_1
        put(1, jc);
        for (int l = 1; l < L0; ++l) {
            const float jn = (2.f * l + 1.f) * ix * jc - jm;
            put(l + 1, jn);
            jm = jc;
            jc = jn;
        }
    } else {
        jc = j0;
    }
    if (L0 >= li) return;
    // l > L0: ratios r_l = j_l / j_{l-1} by the continued fraction
    // r_l = x / (2l + 1 - x r_{l+1}), started 16 orders above the last one needed
    const int top = min(li + 16, kMaxL - 1);
    float rr[kMaxL];
    float rn = 0.f;
    for (int l = top; l > L0; --l) {
        rn = x / (2.f * l + 1.f - x * rn);
        if (l <= li) rr[l] = rn;
    }
    float v = jc;  // j_{L0}
    for (int l = L0 + 1; l <= li; ++l) {
        v *= rr[l];
        put(l, v);
    }
}

// ---------------------------------------------------------------------------
// hm_gemm: block (m tile, shell tile, l); 256 threads = 8 shell groups of 4
// shells x 32 lanes of 2 m each.  C[i][k] (FP64) += the chunk's sum; every
// element has one owner per chunk and the chunks run in order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) hm_gemm(const float* __restrict__ J, const float2* __restrict__ Y, int ch,
                                               int Lp, int K, const int* __restrict__ imin,
                                               const int64_t* __restrict__ joff, double2* __restrict__ C) {
    __shared__ __align__(16) float sJ[kGemmSub][kGemmShells + 4];
    __shared__ float2 sY[kGemmSub][kGemmM + 1];
    const int l = blockIdx.z;
    const int m0 = blockIdx.x * kGemmM;
    if (m0 > l) return;
    const int i_lo = imin[l];
    const int rows = Lp - i_lo + 1;  // shells with l_i >= l
    const int s0 = blockIdx.y * kGemmShells;
    if (s0 >= rows) return;
    const int t = threadIdx.x, lane = t & 31, grp = t >> 5;
    const float* Jl = J + joff[l] * ch;
    const int64_t kb = (int64_t)k_of(l, 0);
    float ar[4][2], ai[4][2], sr[4][2], si[4][2], cr[4][2], ci[4][2];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) ar[a][b] = ai[a][b] = sr[a][b] = si[a][b] = cr[a][b] = ci[a][b] = 0.f;
    for (int j0 = 0; j0 < ch; j0 += kGemmSub) {
        __syncthreads();
        // stage J rows s0..s0+31 and Y columns m0..m0+63 for points j0..j0+63
        for (int e = t; e < kGemmSub * kGemmShells; e += 256) {
            const int sh = e / kGemmSub, jj = e % kGemmSub;
            sJ[jj][sh] = (s0 + sh < rows) ? Jl[(int64_t)(s0 + sh) * ch + j0 + jj] : 0.f;
        }
        for (int e = t; e < kGemmSub * kGemmM; e += 256) {
            const int mm = e / kGemmSub, jj = e % kGemmSub;
            sY[jj][mm] = (m0 + mm <= l) ? Y[(kb + m0 + mm) * ch + j0 + jj] : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll 4
        for (int jj = 0; jj < kGemmSub; ++jj) {
            const float4 jv = *reinterpret_cast<const float4*>(&sJ[jj][grp * 4]);
            const float2 y0 = sY[jj][lane], y1 = sY[jj][lane + 32];
            const float js[4] = {jv.x, jv.y, jv.z, jv.w};
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                ar[a][0] = fmaf(js[a], y0.x, ar[a][0]);
                ai[a][0] = fmaf(js[a], y0.y, ai[a][0]);
                ar[a][1] = fmaf(js[a], y1.x, ar[a][1]);
                ai[a][1] = fmaf(js[a], y1.y, ai[a][1]);
            }
        }
        // Kahan-compensated running sums of the 64-point partial sums
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                float y = ar[a][b] - cr[a][b];
                float tt = sr[a][b] + y;
                cr[a][b] = (tt - sr[a][b]) - y;
                sr[a][b] = tt;
                y = ai[a][b] - ci[a][b];
                tt = si[a][b] + y;
                ci[a][b] = (tt - si[a][b]) - y;
                si[a][b] = tt;
                ar[a][b] = ai[a][b] = 0.f;
            }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int row = s0 + grp * 4 + a;
        if (row >= rows) continue;
        const int i = i_lo + row;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const int m = m0 + lane + 32 * b;
            if (m > l) continue;
            double2& c = C[(int64_t)i * K + kb + m];
            c.x += (double)sr[a][b] - (double)cr[a][b];
            c.y += (double)si[a][b] - (double)ci[a][b];
        }
    }
}

__device__ __forceinline__ float sinc_h(float h) {
    const float h2 = h * h;
    if (h2 < 0.25f) return fmaf(h2, fmaf(h2, fmaf(h2, -1.f / 5040.f, 1.f / 120.f), -1.f / 6.f), 1.f);
    return __fdividef(__sinf(h), h);
}

// ---------------------------------------------------------------------------
// hm_synth: one block per theta row (i, t <= 3i/2); rows[] lists (i, t).
// Dynamic shared memory: P column values [K_i], B and B' (atoms, voxels),
// the 6i roots of unity.
// ---------------------------------------------------------------------------
__global__ void hm_synth(const int2* __restrict__ rows, const double2* __restrict__ Ca, const double2* __restrict__ Cv,
                         int K, const int* __restrict__ lmax, const float2* __restrict__ ab, double step,
                         float vox_s, double cx, double cy, double cz, int use_center, float scale, double origin,
                         float4* __restrict__ grid) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int2 row = rows[blockIdx.x];
    const int i = row.x, t = row.y;
    const int li = lmax[i];
    const int Ki = k_of(li, li) + 1;
    const int nph = 6 * i, h = 3 * i;
    float* sP = reinterpret_cast<float*>(smem);
    float2* sB = reinterpret_cast<float2*>(smem + ((size_t)Ki * 4 + 15) / 16 * 16);
    float2* sBp = sB + (li + 1);
    float2* sBv = sBp + (li + 1);
    float2* sBpv = sBv + (li + 1);
    float2* sW = sBpv + (li + 1);
    const bool vox = Cv != nullptr;
    float st, ct;
    sincospif((float)t / (float)h, &st, &ct);
    // Legendre column m per thread
    for (int m = threadIdx.x; m <= li; m += blockDim.x) {
        float pmm = 0.28209479177387814347f;
        for (int mm = 1; mm <= m; ++mm) pmm = -sqrtf((2.f * mm + 1.f) / (2.f * mm)) * st * pmm;
        float p2 = 0.f, p1 = pmm;
        sP[k_of(m, m)] = p1;
        for (int l = m + 1; l <= li; ++l) {
            const float2 c = ab[k_of(l, m)];
            const float p0 = c.x * fmaf(ct, p1, -c.y * p2);
            sP[k_of(l, m)] = p0;
            p2 = p1;
            p1 = p0;
        }
    }
    for (int n = threadIdx.x; n < nph; n += blockDim.x) {
        float sw, cw;
        sincospif(2.f * (float)n / (float)nph, &sw, &cw);
        sW[n] = make_float2(cw, sw);
    }
    __syncthreads();
    // B_m = 4 pi sum_l i^l P_lm C_lm ; B'_m = 4 pi sum_l i^l P_lm conj(C_lm)
    const double2* Cai = Ca + (int64_t)i * K;
    const double2* Cvi = vox ? Cv + (int64_t)i * K : nullptr;
    for (int m = threadIdx.x; m <= li; m += blockDim.x) {
        float br = 0.f, bi = 0.f, pr = 0.f, pi_ = 0.f;
        float vr = 0.f, vi = 0.f, qr = 0.f, qi = 0.f;
        for (int l = m; l <= li; ++l) {
            const int k = k_of(l, m);
            const float p = sP[k];
            const double2 cd = Cai[k];
            const float2 c = make_float2((float)cd.x, (float)cd.y);
            // i^l (c.x + i c.y) and i^l (c.x - i c.y)
            float ar, ai, er, ei;
            switch (l & 3) {
                case 0: ar = c.x; ai = c.y; er = c.x; ei = -c.y; break;
                case 1: ar = -c.y; ai = c.x; er = c.y; ei = c.x; break;
                case 2: ar = -c.x; ai = -c.y; er = -c.x; ei = c.y; break;
                default: ar = c.y; ai = -c.x; er = -c.y; ei = -c.x; break;
            }
            br = fmaf(p, ar, br);
            bi = fmaf(p, ai, bi);
            pr = fmaf(p, er, pr);
            pi_ = fmaf(p, ei, pi_);
            if (vox) {
                const double2 dd = Cvi[k];
                const float2 d = make_float2((float)dd.x, (float)dd.y);
                switch (l & 3) {
                    case 0: ar = d.x; ai = d.y; er = d.x; ei = -d.y; break;
                    case 1: ar = -d.y; ai = d.x; er = d.y; ei = d.x; break;
                    case 2: ar = -d.x; ai = -d.y; er = -d.x; ei = d.y; break;
                    default: ar = d.y; ai = -d.x; er = -d.y; ei = -d.x; break;
                }
                vr = fmaf(p, ar, vr);
                vi = fmaf(p, ai, vi);
                qr = fmaf(p, er, qr);
                qi = fmaf(p, ei, qi);
            }
        }
        sB[m] = make_float2(kFourPi * br, kFourPi * bi);
        sBp[m] = make_float2(m > 0 ? kFourPi * pr : 0.f, m > 0 ? kFourPi * pi_ : 0.f);
        if (vox) {
            sBv[m] = make_float2(kFourPi * vr, kFourPi * vi);
            sBpv[m] = make_float2(m > 0 ? kFourPi * qr : 0.f, m > 0 ? kFourPi * qi : 0.f);
        }
    }
    __syncthreads();
    const float qI = (float)((double)i * step);
    const int64_t base = shell_base(i);
    for (int p = threadIdx.x; p < nph; p += blockDim.x) {
        float ar = 0.f, ai = 0.f, vr = 0.f, vi = 0.f;
        int idx = 0;  // (m p) mod 6i
        for (int m = 0; m <= li; ++m) {
            const float2 w = sW[idx];
            const float2 b = sB[m], bp = sBp[m];
            // b w + bp conj(w)
            ar += b.x * w.x - b.y * w.y + bp.x * w.x + bp.y * w.y;
            ai += b.x * w.y + b.y * w.x + bp.y * w.x - bp.x * w.y;
            if (vox) {
                const float2 c = sBv[m], cp = sBpv[m];
                vr += c.x * w.x - c.y * w.y + cp.x * w.x + cp.y * w.y;
                vi += c.x * w.y + c.y * w.x + cp.y * w.x - cp.x * w.y;
            }
            idx += p;  // idx, p < 6i
            if (idx >= nph) idx -= nph;
        }
        float sp, cp;
        sincospif((float)p / (float)h, &sp, &cp);
        const float qx = qI * st * cp, qy = qI * st * sp, qz = qI * ct;
        if (vox) {
            const float f = vox_s * sinc_h(0.5f * qx * vox_s) * vox_s * sinc_h(0.5f * qy * vox_s) * vox_s *
                            sinc_h(0.5f * qz * vox_s);
            ar = fmaf(f, vr, ar);
            ai = fmaf(f, vi, ai);
        }
        float2 F = make_float2(ar * scale, ai * scale);
        if (use_center) {
            double s1, c1;
            sincos((double)qx * cx + (double)qy * cy + (double)qz * cz, &s1, &c1);
            F = make_float2((float)(F.x * c1 - F.y * s1), (float)(F.x * s1 + F.y * c1));
        }
        grid[base + (int64_t)t * nph + p] = make_float4(F.x, F.y, 0.f, 0.f);
        // Friedel: the antipode (3i - t, p + 3i) holds the conjugate (the
        // equator row is its own mirror and is written once per cell)
        if (2 * t != h) {
            const int pm = p < h ? p + h : p - h;
            grid[base + (int64_t)(h - t) * nph + pm] = make_float4(F.x, -F.y, 0.f, 0.f);
        }
    }
    if (i == 1 && t == 0 && threadIdx.x == 0) grid[0] = make_float4((float)origin, 0.f, 0.f, 0.f);
}

}  // namespace

int harmonic_max_l() { return kMaxL - 17; }

cudaError_t launch_harmonic_chunk(cudaStream_t s, const HarmonicArgs& a, bool voxels, int64_t chunk_off,
                                  double2* C) {
    const int ch = a.ch;
    hm_basis<<<dim3((ch + 127) / 128, a.LM + 1), 128, 0, s>>>(a.pts, a.n, chunk_off, ch, a.LM, a.ab, a.Y);
    if (voxels)
        hm_bessel<true><<<dim3((ch + 127) / 128, a.Lp), 128, 0, s>>>(a.pts, a.n, chunk_off, ch, a.Lp, a.step, a.lmax,
                                                                     a.imin, a.joff, a.aff, a.J);
    else
        hm_bessel<false><<<dim3((ch + 127) / 128, a.Lp), 128, 0, s>>>(a.pts, a.n, chunk_off, ch, a.Lp, a.step,
                                                                      a.lmax, a.imin, a.joff, a.aff, a.J);
    const int mt = (a.LM + kGemmM) / kGemmM;
    const int st = (a.Lp + kGemmShells - 1) / kGemmShells;
    hm_gemm<<<dim3(mt, st, a.LM + 1), 256, 0, s>>>(a.J, a.Y, ch, a.Lp, a.K, a.imin, a.joff, C);
    return cudaGetLastError();
}

cudaError_t launch_harmonic_synth(cudaStream_t s, const HarmonicSynth& a) {
    // one launch; dynamic shared memory sized for the outermost shell
    const int li = a.lmax_host_outer;
    const int nph = 6 * a.Lp;
    const size_t smem = ((size_t)((li + 1) * (li + 2) / 2) * 4 + 15) / 16 * 16 + (size_t)4 * (li + 1) * sizeof(float2) +
                        (size_t)nph * sizeof(float2);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(hm_synth, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    hm_synth<<<a.n_rows, 256, smem, s>>>(a.rows, a.Ca, a.Cv, a.K, a.lmax, a.ab, a.step, a.vox_s, a.cx, a.cy, a.cz,
                                         a.use_center, a.scale, a.origin, a.grid);
    return cudaGetLastError();
}

}  // namespace dpx
