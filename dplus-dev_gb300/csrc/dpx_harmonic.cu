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
// |r_j| about the centre: beyond it j_l(x) is below 1e-7 of its peak.
//
// Radial bins.  Points are grouped by radius into bins of width
// delta = 0.7 / q_max (and, for atoms, by ion); within bin b (centre r_b) the
// radial factor is a degree-5 polynomial in u = (r - r_b) / (delta / 2):
//   j_l(q_i r) = sum_n T_n(i, b, l) u^n    (interpolation at 6 Chebyshev nodes,
//                                           error below 2e-8 for q <= q_max)
// so that C_lm(q_i) = sum_groups F_g(q_i) sum_n T_n(i, b_g, l) M_g[n][lm] with the
// per-group moments M_g[n][lm] = sum_{j in g} w_j u_j^n Pbar_lm(cos theta_j)
// e^{-i m phi_j}.  A point costs 6 (l_max+1)(l_max+2)/2 multiply-adds whatever
// the number of shells, and the radial functions are evaluated once per
// (shell, bin, node) instead of once per (shell, point).
//
// Kernels:
//   hm_nodes     j_l at the Chebyshev nodes of every (shell, bin), FP64   } once per plan
//   hm_fit       T_n(i, b, l) from the node values (inverse Vandermonde)  } (launch_radial_tables)
//   hm_moments   per unit of <= 1024 points of one group: M_unit[n][k] on the
//                tensor cores (split TF32, FP32 sums), the basis values in
//                registers by scaled Legendre recurrences
//   hm_groups    M_g = sum of its units, compensated FP32
//   hm_contract  C[i][k] = sum_g F_g(q_i) sum_n T_n M_g[n][k], compensated FP32
//   hm_synth     per theta row t <= 3i/2: the B_m of both exponentials, the 6i
//                cells by a table of 6i-th roots of unity, the voxel form
//                factor prod_a s sinc(q_a s / 2) on the solvent part (a box of
//                n voxels is exactly the sum of its voxels), the centring
//                phase e^{i q.c} in double-float, the Friedel mirror row and
//                the rows' phi-spline derivatives.
#include "dpx_internal.h"

#include <atomic>
#include <mutex>
#include "dpx_spline.cuh"

#include <cstdint>
#include <cuda_fp16.h>

namespace dpx {
namespace {

constexpr float kFourPi = 12.566370614359172954f;
constexpr int kNodes = 6;       // Chebyshev nodes per bin = polynomial degree + 1
constexpr int kMaxL = 192;      // local recurrence arrays

__device__ __forceinline__ int k_of(int l, int m) { return l * (l + 1) / 2 + m; }
__device__ __forceinline__ int l_of(int k) {
    int l = (int)((sqrtf(8.f * (float)k + 1.f) - 1.f) * 0.5f);
    while (k_of(l + 1, 0) <= k) ++l;
    while (k_of(l, 0) > k) --l;
    return l;
}

// ---------------------------------------------------------------------------
// hm_nodes: thread (shell i >= 1, bin b, node c).  j_l(x), l <= l_i, in FP64:
// upward recurrence for l <= floor(x), the continued fraction
// r_l = x / (2l + 1 - x r_{l+1}) (started 16 orders above) for the ratios above.
// Jn[((i * nbins + b) * kNodes + c) * (LM + 1) + l].
// ---------------------------------------------------------------------------
__device__ void hm_nodes(int Lp, int nbins, int LM, double step, double delta, const int* __restrict__ lmax,
                         const double* __restrict__ nodes, double* __restrict__ Jn, int64_t e) {
    const int64_t total = (int64_t)Lp * nbins * kNodes;
    if (e >= total) return;
    const int c = (int)(e % kNodes);
    const int b = (int)((e / kNodes) % nbins);
    const int i = (int)(e / ((int64_t)kNodes * nbins)) + 1;
    const int li = lmax[i];
    double* out = Jn + (((int64_t)i * nbins + b) * kNodes + c) * (LM + 1);
    const double x = (double)i * step * ((b + 0.5) * delta + nodes[c] * 0.5 * delta);
    if (x < 1e-8) {
        out[0] = 1.0;
        for (int l = 1; l <= li; ++l) out[l] = 0.0;
        return;
    }
    double s, co;
    sincos(x, &s, &co);
    const double ix = 1.0 / x;
    const double j0 = s * ix;
    out[0] = j0;
    const int L0 = min((int)x, li);
    double jm = j0, jc = j0;
    if (L0 >= 1) {
        jc = (j0 - co) * ix;
        out[1] = jc;
        for (int l = 1; l < L0; ++l) {
            const double jn = (2.0 * l + 1.0) * ix * jc - jm;
            out[l + 1] = jn;
            jm = jc;
            jc = jn;
        }
    }
    if (L0 >= li) return;
    const int top = min(li + 16, kMaxL - 1);
    double rr[kMaxL];
    double rn = 0.0;
    for (int l = top; l > L0; --l) {
        rn = x / (2.0 * l + 1.0 - x * rn);
        if (l <= li) rr[l] = rn;
    }
    double v = jc;
    for (int l = L0 + 1; l <= li; ++l) {
        v *= rr[l];
        out[l] = v;
    }
}

// hm_fit: thread (shell i >= 1, bin b, l <= l_i): T[((i nbins + b)(LM+1) + l) * 8 + n].
__device__ void hm_fit(int Lp, int nbins, int LM, const int* __restrict__ lmax, const double* __restrict__ vinv,
                       const double* __restrict__ Jn, float* __restrict__ T, int64_t e) {
    const int64_t total = (int64_t)Lp * nbins * (LM + 1);
    if (e >= total) return;
    const int l = (int)(e % (LM + 1));
    const int b = (int)((e / (LM + 1)) % nbins);
    const int i = (int)(e / ((int64_t)(LM + 1) * nbins)) + 1;
    float* out = T + (((int64_t)i * nbins + b) * (LM + 1) + l) * 8;
    if (l > lmax[i]) {
        for (int n = 0; n < 8; ++n) out[n] = 0.f;
        return;
    }
    const double* jn = Jn + (((int64_t)i * nbins + b) * kNodes) * (LM + 1) + l;
    double v[kNodes];
    for (int c = 0; c < kNodes; ++c) v[c] = jn[(int64_t)c * (LM + 1)];
    for (int n = 0; n < kNodes; ++n) {
        double t = 0.0;
        for (int c = 0; c < kNodes; ++c) t += vinv[n * kNodes + c] * v[c];
        out[n] = (float)t;
    }
    out[6] = out[7] = 0.f;
}

// ---------------------------------------------------------------------------
// hm_moments: MP[u][n][k] (FP32) = sum over the points of unit u of
// w u^n Pbar_lm(cos theta) e^{-i m phi}, k = (l, m), n < 6, on the tensor cores.
//
// One warp per (unit, pair of column quartets): quartet q holds the orders
// m = 4q .. 4q+3, and the pair {q, Q-1-q} gives every warp about l_max + 2
// rows of work.  Per quartet the warp walks the unit's points in chunks of 32
// (four k-steps of 8) and, per order l, issues
//   D[16 x 8] += A[16 x 8] B[8 x 8]     (mma.sync m16n8k8, TF32 in, FP32 out)
// with A the weights (rows n: w u^n rounded to TF32; rows 8 + n: the
// remainder, so that both halves of the split weight are applied) and B the
// basis values of the chunk's points (columns: the quartet's 4 orders m x
// {re, im}), B split the same way over two MMAs: every product carries the
// hi*hi + hi*lo + lo*hi + lo*lo terms of the FP32 operands.  Lane (g, t)
// builds the basis values of column g (order m0 + g/2, component g%2) at the
// points 8j + t and 8j + t + 4 of k-step j: eight Legendre recurrences in
// registers.  The recurrence is scaled, q_l = Pbar_lm / r_lm with
// r_lm = prod_{j=m+1..l} a_jm / 2, so that one step is
//   q_l = 2x q_{l-1} - c_lm q_{l-2},   c_lm = 4 b_lm / a_{l-1,m}
// (cr[k] = {c_lm, r_lm}); r_lm is applied once per moment at the store.  The
// start q_m = nmm[m] (-sin theta)^m e^{-i m phi} = nmm[m] z^m with
// z = (-x + i y) / r (binary powering: no angles).  The D rows of lane (g, t),
// n = g (hi and remainder rows summed), columns 2t, 2t+1, are the complex
// moment of order m0 + t; they are summed over the chunks in shared memory.
// ---------------------------------------------------------------------------
constexpr int kChunk = 32;  // points per chunk: four k-steps of the m16n8k8 MMA

__device__ __forceinline__ uint32_t tf32_rna(float v) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Packed FP32 pairs (the f32x2 arithmetic of sm_100 and later): two chains
// per instruction, each lane of the pair an IEEE FP32 operation.
typedef unsigned long long f2x;
__device__ __forceinline__ f2x pk2(float a, float b) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(f2x v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
    f2x r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
    f2x r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x sub2(f2x a, f2x b) {
    f2x r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x add2(f2x a, f2x b) {
    f2x r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ float2 cpow(float2 z, int e) {  // z^e, e >= 0, by binary powering
    float2 r = make_float2(1.f, 0.f);
    for (; e > 0; e >>= 1) {
        if (e & 1) r = cmulf(r, z);
        z = cmulf(z, z);
    }
    return r;
}

__device__ __forceinline__ float2 shfl2(float2 v, int src) {
    return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// One order l of a quartet: the eight recurrences in four packed pairs (the
// pair of k-step j = the points 8j + t and 8j + t + 4; q_old holds q_{l-2} on
// entry and q_l on exit, q_new holds q_{l-1}), the TF32 split of the basis
// values (the high part by truncation, the exact remainder), then the chunk's
// MMAs into the running sums sDl[lane].  PRO: the first four orders, where a
// column starts (q_m = its start value) or has not started yet.
template <bool PRO>
__device__ __forceinline__ void moment_order(int l, int m, bool col_ok, int kc, const float2* __restrict__ cr,
                                             f2x (&q_old)[4], const f2x (&q_new)[4], const f2x (&x2)[4],
                                             const f2x (&st)[4], const uint32_t (&A)[4][4], float2* sDl,
                                             bool drow, int lane) {
    float cl;
    if (PRO) cl = (col_ok && l >= m + 2) ? __ldg(&cr[kc].x) : 0.f;
    else cl = __ldg(&cr[kc].x);
    const f2x ncl = pk2(-cl, -cl);
    const bool start = PRO && col_ok && l == m;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const f2x v = fma2(x2[j], q_new[j], mul2(ncl, q_old[j]));
        q_old[j] = start ? st[j] : v;
    }
    // one accumulator per k-step: four independent chains of two MMAs
    float d[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
    if (drow) {
        const float2 prev = sDl[lane];
        d[0][0] = prev.x;
        d[0][1] = prev.y;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float v0, v1;
        upk2(q_old[j], v0, v1);
        const uint32_t h0 = __float_as_uint(v0) & 0xffffe000u, h1 = __float_as_uint(v1) & 0xffffe000u;
        float r0, r1;
        upk2(sub2(q_old[j], pk2(__uint_as_float(h0), __uint_as_float(h1))), r0, r1);
        mma_tf32(d[j], A[j], h0, h1);
        mma_tf32(d[j], A[j], __float_as_uint(r0), __float_as_uint(r1));
    }
    if (drow) {
        f2x s[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) s[j] = add2(pk2(d[j][0], d[j][1]), pk2(d[j][2], d[j][3]));
        float re, im;
        upk2(add2(add2(s[0], s[1]), add2(s[2], s[3])), re, im);
        sDl[lane] = make_float2(re, im);
    }
}

// FP16 variant of one order (the H kernel below): the basis values are the
// true Pbar_lm e^{-i m phi} times 2^11 (the scaled recurrence times r_lm 2^11:
// both FP16 halves stay in the normal range), split into the FP16 value (the
// FP32 value truncated to 11 significant bits) and the FP16 remainder; the
// pairs are the points (2t, 2t + 1) and (2t + 8, 2t + 9) of the k-steps of 16
// points, one f16x2 register each, and each k-step takes two m16n8k16 MMAs
// (value and remainder against the weights' value and remainder rows).
__device__ __forceinline__ void mma_f16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t h2pack(float x0, float x1) {  // x0 in the low half (the lower k)
    const __half2 h = __floats2half2_rn(x0, x1);
    return *reinterpret_cast<const uint32_t*>(&h);
}

template <bool PRO>
__device__ __forceinline__ void moment_order_h(int l, int m, bool col_ok, int kc, const float2* __restrict__ cr,
                                               f2x (&q_old)[4], const f2x (&q_new)[4], const f2x (&x2)[4],
                                               const f2x (&st)[4], const uint32_t (&A)[2][4], float2* sDl,
                                               bool drow, int lane) {
    const float2 cv = col_ok ? __ldg(&cr[kc]) : make_float2(0.f, 0.f);
    const float cl = (PRO && l < m + 2) ? 0.f : cv.x;
    const f2x ncl = pk2(-cl, -cl);
    const bool start = PRO && col_ok && l == m;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const f2x v = fma2(x2[j], q_new[j], mul2(ncl, q_old[j]));
        q_old[j] = start ? st[j] : v;
    }
    const float rs = cv.y * 2048.f;  // r_lm 2^11 (1 at l = m)
    const f2x rs2 = pk2(rs, rs);
    uint32_t Bh[4], Bl[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const f2x v = mul2(q_old[j], rs2);
        float v0, v1;
        upk2(v, v0, v1);
        const float h0 = __uint_as_float(__float_as_uint(v0) & 0xffffe000u);
        const float h1 = __uint_as_float(__float_as_uint(v1) & 0xffffe000u);
        float r0, r1;
        upk2(sub2(v, pk2(h0, h1)), r0, r1);
        Bh[j] = h2pack(h0, h1);
        Bl[j] = h2pack(r0, r1);
    }
    // one accumulator per k-step: two independent chains of two MMAs, started
    // at zero (the running sum is added in FP32 afterwards: the FP16 MMAs'
    // accumulation rounds less finely, measured 2.9e-6 against 1.5e-6 for the
    // bench subunit's I(q) when the running sum went through them)
    float d[2][4];
#pragma unroll
    for (int j = 0; j < 2; ++j) d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
    const float2 prev = drow ? sDl[lane] : make_float2(0.f, 0.f);  // loaded while the MMAs run
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        mma_f16(d[j], A[j], Bh[2 * j], Bh[2 * j + 1]);
        mma_f16(d[j], A[j], Bl[2 * j], Bl[2 * j + 1]);
    }
    if (drow) {
        const f2x s0 = add2(pk2(d[0][0], d[0][1]), pk2(d[0][2], d[0][3]));
        const f2x s1 = add2(pk2(d[1][0], d[1][1]), pk2(d[1][2], d[1][3]));
        float re, im;
        upk2(add2(pk2(prev.x, prev.y), add2(s0, s1)), re, im);
        sDl[lane] = make_float2(re, im);
    }
}

template <bool H, bool PRO>
__device__ __forceinline__ void order_step(int l, int m, bool col_ok, int kc, const float2* __restrict__ cr,
                                           f2x (&q_old)[4], const f2x (&q_new)[4], const f2x (&x2)[4],
                                           const f2x (&st)[4], const uint32_t (&A)[4][4], float2* sDl, bool drow,
                                           int lane) {
    if (H)
        moment_order_h<PRO>(l, m, col_ok, kc, cr, q_old, q_new, x2, st,
                            *reinterpret_cast<const uint32_t(*)[2][4]>(&A[0][0]), sDl, drow, lane);
    else
        moment_order<PRO>(l, m, col_ok, kc, cr, q_old, q_new, x2, st, A, sDl, drow, lane);
}

// H = false: TF32 operands (moment_order); H = true: FP16 operands
// (moment_order_h), the weights w u^n scaled by 2^(14 - e) per unit (2^e above
// the unit's largest |w|), the moments stored times 2^(e - 25).
template <bool H>
__device__ void hm_moments(const float4* __restrict__ pts, const int4* __restrict__ units, int K, float delta,
                           const int* __restrict__ lmb, const float2* __restrict__ cr, const float* __restrict__ nmm,
                           float2* __restrict__ MP, int bx, int by) {
    extern __shared__ __align__(16) unsigned char smem[];
    float2* sD = reinterpret_cast<float2*>(smem);  // per quartet [(l - m0) * 24 + lane], lanes < 24
    const int lane = threadIdx.x;
    const int g = lane >> 2, t = lane & 3;
    const int4 un = units[bx];
    const int LM = lmb[un.z];    // the orders of the unit's bin
    const int Q = (LM + 4) / 4;  // quartets
    if (by >= (Q + 1) / 2) return;
    const int nq = (Q - 1 - by > by) ? 2 : 1;
    const int m0a = 4 * by, m0b = 4 * (Q - 1 - by);
    const int nla = LM - m0a + 1, nlb = nq == 2 ? LM - m0b + 1 : 0;
    const float rb = (un.z + 0.5f) * delta, ih = 2.f / delta;
    const bool drow = lane < 24;  // D rows n = g < 6
    for (int e = lane; e < (nla + nlb) * 24; e += 32) sD[e] = make_float2(0.f, 0.f);
    __syncwarp();
    float wsc = 1.f, wback = 1.f;
    if (H) {  // the unit's largest |w|: the FP16 weights' scale
        float wm = 0.f;
        for (int j = lane; j < un.y; j += 32) wm = fmaxf(wm, fabsf(__ldg(&pts[un.x + j]).w));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, o));
        int e = 0;
        frexpf(wm, &e);
        wsc = ldexpf(1.f, 14 - e);
        wback = ldexpf(1.f, e - 25);
    }

    for (int c0 = 0; c0 < un.y; c0 += kChunk) {
        // ---- point c0 + lane: geometry and the powers z^m0 of the pair's quartets ----
        float ct = 1.f, u = 0.f, w = 0.f;
        float2 z = make_float2(0.f, 0.f);
        if (c0 + lane < un.y) {
            const float4 P = pts[un.x + c0 + lane];
            const float r = sqrtf(fmaf(P.z, P.z, fmaf(P.x, P.x, P.y * P.y)));
            if (r > 0.f) {
                const float ir = 1.f / r;
                ct = P.z * ir;
                z = make_float2(-P.x * ir, P.y * ir);
            }
            u = (r - rb) * ih;
            w = P.w;
        }
        const float2 zq0 = cpow(z, m0a);
        const float2 zq1 = nq == 2 ? cpow(z, m0b) : make_float2(0.f, 0.f);
        // ---- the lane's eight points (pair j, member h: 8j + t + 4h for TF32, the
        // m16n8k8 fragment; 16 (j / 2) + 2t + 8 (j % 2) + h for FP16, m16n8k16):
        // recurrence inputs, weight fragments ----
        f2x x2[4];
        uint32_t A[4][4];  // H: [k-step][a0..a3], k-steps 0, 1
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float xx[2], wh2[2], wl2[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int src = H ? 16 * (j >> 1) + 2 * t + 8 * (j & 1) + h : 8 * j + t + 4 * h;
                xx[h] = 2.f * __shfl_sync(0xffffffffu, ct, src);
                const float us = __shfl_sync(0xffffffffu, u, src);
                float wv = __shfl_sync(0xffffffffu, w, src);
                // weight w u^n of row n = g, split into the value (row g) and remainder (row g + 8)
                if (g >= 6) wv = 0.f;
                for (int n = 0; n < g; ++n) wv *= us;
                if (H) {
                    wv *= wsc;
                    const float vh = __half2float(__float2half_rn(wv));
                    wh2[h] = vh;
                    wl2[h] = wv - vh;
                } else {
                    const uint32_t wh = tf32_rna(wv);
                    A[j][2 * h] = wh;                                          // a0 / a2: row g
                    A[j][2 * h + 1] = __float_as_uint(wv - __uint_as_float(wh));  // a1 / a3: row g + 8
                }
            }
            if (H) {  // a0 / a1: rows g, g + 8 at the k-step's points 2t, 2t + 1; a2 / a3 at 2t + 8, 2t + 9
                A[j >> 1][2 * (j & 1)] = h2pack(wh2[0], wh2[1]);
                A[j >> 1][2 * (j & 1) + 1] = h2pack(wl2[0], wl2[1]);
            }
            x2[j] = pk2(xx[0], xx[1]);
        }
        // ---- the pair's quartets ----
#pragma unroll 1
        for (int qi = 0; qi < nq; ++qi) {
            const int m0 = qi == 0 ? m0a : m0b;
            const float2 zq = qi == 0 ? zq0 : zq1;
            const int c = g >> 1;  // this lane's column m0 + c, component g & 1
            const int m = m0 + c;
            const bool col_ok = m <= LM;
            const float nm = col_ok ? nmm[m] : 0.f;
            f2x st[4], qa_[4], qb_[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float sv[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int src = H ? 16 * (j >> 1) + 2 * t + 8 * (j & 1) + h : 8 * j + t + 4 * h;
                    const float2 zp = shfl2(z, src);
                    float2 zm = shfl2(zq, src);  // z^m0 of the point, times z^c
                    if (c >= 1) zm = cmulf(zm, zp);
                    if (c >= 2) zm = cmulf(zm, zp);
                    if (c >= 3) zm = cmulf(zm, zp);
                    sv[h] = nm * ((g & 1) ? zm.y : zm.x);
                }
                st[j] = pk2(sv[0], sv[1]);
                qa_[j] = 0ull;
                qb_[j] = 0ull;
            }
            float2* sDq = sD + (qi == 0 ? 0 : nla * 24);
            int kc = col_ok ? m0 * (m0 + 1) / 2 + m : 0;  // k(l, m) at l = m0 (read once l >= m + 2)
            int l = m0;
            // orders m0 .. m0 + 3: the columns start
#pragma unroll
            for (int s2 = 0; s2 < 2; ++s2) {
                if (l <= LM) order_step<H, true>(l, m, col_ok, kc, cr, qa_, qb_, x2, st, A, sDq + (l - m0) * 24, drow, lane);
                if (col_ok) kc += l + 1;
                ++l;
                if (l <= LM) order_step<H, true>(l, m, col_ok, kc, cr, qb_, qa_, x2, st, A, sDq + (l - m0) * 24, drow, lane);
                if (col_ok) kc += l + 1;
                ++l;
            }
            // the rest, two orders per iteration
            for (; l + 1 <= LM; l += 2) {
                order_step<H, false>(l, m, col_ok, kc, cr, qa_, qb_, x2, st, A, sDq + (l - m0) * 24, drow, lane);
                if (col_ok) kc += l + 1;
                order_step<H, false>(l + 1, m, col_ok, kc, cr, qb_, qa_, x2, st, A, sDq + (l + 1 - m0) * 24, drow, lane);
                if (col_ok) kc += l + 2;
            }
            if (l <= LM) order_step<H, false>(l, m, col_ok, kc, cr, qa_, qb_, x2, st, A, sDq + (l - m0) * 24, drow, lane);
        }
    }
    __syncwarp();
    // ---- store: lane (g < 6, t) holds the moment n = g of order m0 + t ----
    for (int qi = 0; qi < nq; ++qi) {
        const int m0 = qi == 0 ? m0a : m0b;
        const int mo = m0 + t;
        if (!drow || mo > LM) continue;
        const float2* sDq = sD + (qi == 0 ? 0 : nla * 24);
        float2* out = MP + ((int64_t)bx * kNodes + g) * K;
        int k = mo * (mo + 1) / 2 + mo;
        for (int l = mo; l <= LM; ++l) {
            const float2 v = sDq[(l - m0) * 24 + lane];
            const float sc = H ? wback : __ldg(&cr[k].y);
            out[k] = make_float2(v.x * sc, v.y * sc);
            k += l + 1;
        }
    }
}

// ---------------------------------------------------------------------------
// hm_moments_tc: the same moments MP[u][n][k] on the fifth-generation tensor
// cores: tcgen05.mma kind::f16 with FP16 operands and FP32 accumulators in
// tensor memory.  Per tile of 64 points and 128 rows (a row = one (l, m) and
// re or im):
//   D[row][col] += A[row][p] B[col][p]            (M = 128, N = 16, K = 16 per MMA)
// A = the rows' basis values at the 64 points, written into tensor memory by
// the producer warps (tcgen05.st), twice: the FP16 value (hi) and the FP16
// remainder (lo), one MMA each per K-step; B = the weights w u^n of the points
// in shared memory (K-major, 128-byte swizzle): rows n < 6 hi, rows 6 + n lo,
// rows 12..15 zero.  So D[row][n] + D[row][6 + n] carries all four products
// hi*hi + hi*lo + lo*hi + lo*lo of the FP32 operands (about 22 bits), and the
// basis values never pass through shared memory.  The basis values are the
// orthonormal Pbar_lm(cos theta) e^{-i m phi} (at most about 5.3 in magnitude
// for l <= 175), the scaled recurrence of hm_moments times r_lm 2^11; the
// weights are scaled by 2^(14 - e) per unit, 2^e above the unit's largest |w|:
// both halves of both operands stay in the FP16 normal range (the remainders
// too, down to operands 2^-14 of their scale), and the epilogue multiplies by
// 2^(e - 25).
//
// CTA = 4 producer warps, 1 warp that owns the tensor memory (all 512
// columns: two A slots of 64 columns, 24 accumulator tiles of 16) and issues
// the MMAs from one thread, and 4 drain warps.  Producer warp w writes tensor-memory lanes
// 32w .. 32w + 31 of a tile: two consecutive steps (lanes 32w + 16h), in
// each the rows of one octet of orders m = 8o + g (lane 16h + g: re,
// 16h + 8 + g: im); thread (g, t4) holds its row pair at the points
// 16 rep + 4 t4 + i (the 16x256b fragment: two FP16 points per register).
// Step d of octet o is l = m + d for every order of the octet, so the eight
// recurrences of a warp start together (one start per octet, from the
// per-chunk tables z^(8o) and z^g: z^m = z^(8o) z^g), and an order's last
// l = LM ends its row early (zeros after it).  The unit's steps (octets end
// to end) are cut evenly over the 4 P producer slots of its P CTAs; a slot
// that starts inside an octet runs the recurrences silently up to its first
// step.  Pipeline: producer slot fill -> mbarrier full[s] (128 arrivals) ->
// MMA thread issues the tile's 8 MMAs (the tile's accumulator restarts every
// chunk) and commits to empty[s] and done[tile] -> producers refill slot s;
// the four drain warps (warp w reads tensor-memory lanes 32 (w % 4) ..) add the
// tile into FP32 sums in shared memory (round to nearest) and arrive on
// drained[tile], which the tile's next MMAs wait for.  A chain of 8 MMAs per
// accumulator: the tensor cores' accumulation over a whole unit of 1,024
// points (128 MMAs) measured 2.6e-6 of the largest amplitude on voxel leaves,
// against 7e-7 for the mma.sync kernel.  Every wait is bounded (kTcWaitLimit
// polls); a wait that gives up sets g_tc_fault and the CTA drains its MMAs,
// frees tensor memory and returns.
// ---------------------------------------------------------------------------
constexpr int kTcProducers = 4;
constexpr int kTcMmaWarp = kTcProducers;              // warp 4: tensor memory and the MMAs
constexpr int kTcDrainers = 4;                        // warps 5..8: accumulator drains
constexpr int kTcThreads = 32 * (kTcProducers + 1 + kTcDrainers);
constexpr int kTcChunk = 64;                          // points per tile
constexpr int kTcTiles = kTcSlotSteps / 2;            // accumulator tiles
constexpr int kTcUnit = 1024;                         // points per unit at most
constexpr int kTcOctets = kMaxL / 8 + 1;
constexpr uint32_t kTcCols = 512;                     // tensor-memory columns held
constexpr uint32_t kTcAcc0 = 128;                     // first accumulator column
constexpr int kTcWaitLimit = 1 << 22;
constexpr float kTcBasisScale = 2048.f;    // 2^11
constexpr int kTcWeightExp = 14;           // weights scaled to below 2^14
static_assert(kTcAcc0 + 16 * kTcTiles <= kTcCols, "accumulators fit tensor memory");
// shared memory from a 1024-byte aligned base
constexpr size_t kTcOffP = (size_t)kTcUnit / kTcChunk * 2048;           // weights: 16 chunks x 2 KB
constexpr size_t kTcOffZ8 = kTcOffP + (size_t)kTcUnit * sizeof(float4);  // points
constexpr size_t kTcOffZg = kTcOffZ8 + (size_t)kTcOctets * kTcChunk * sizeof(float2);  // z^(8o) per point
constexpr size_t kTcOffAcc = kTcOffZg + (size_t)8 * kTcChunk * sizeof(float2);         // z^g per point
constexpr size_t kTcOffBar = kTcOffAcc + (size_t)kTcTiles * 128 * kNodes * sizeof(float);  // sums [tile][row][n]
constexpr int kTcBars = 4 + 2 * kTcTiles;  // full[2], empty[2], done[tiles], drained[tiles]
constexpr size_t kTcSmemUse = 1024 + kTcOffBar + (size_t)kTcBars * 8 + 16;
// requested per CTA: more than half of an SM's shared memory, so that one CTA
// (which holds all of tensor memory) runs per SM
constexpr size_t kTcSmemLaunch = 150 * 1024;
static_assert(kTcSmemUse <= kTcSmemLaunch, "tensor-core moments shared memory");

__device__ unsigned int g_tc_fault;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
// Waits for the completion of the barrier's phase of this parity; false when
// kTcWaitLimit polls pass first.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
    const uint32_t a = smem_u32(b);
    for (int it = 0; it < kTcWaitLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void producers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(32 * kTcProducers) : "memory"); }

// 16 lanes x 256 bits, repeated over 4 column groups: register 4r + j of thread
// (g, t4) goes to lane base + g + 8 (j / 2), column 8r + 2 t4 + (j % 2).
__device__ __forceinline__ void tmem_st_16x256b_x4(uint32_t taddr, const uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.16x256b.x4.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}
// 32 lanes x 32 bits, 16 columns: thread i reads lane base + i.
__device__ __forceinline__ void tmem_ld_32x32b_x16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}
// D[tmem] (+)= A[tmem] B[smem descriptor]
__device__ __forceinline__ void mma_f16_ts(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
        "r"(a), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(b))
                 : "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1,024 bytes apart (start address and offsets in 16-byte units).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// Instruction descriptor of kind::f16: FP32 accumulator, FP16 A and B, both
// K-major, N = 16, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

// Weight w u^n of chunk point p (< 64) in row r of the swizzled B tile.
__device__ __forceinline__ void tc_put_weight(unsigned char* tile, int r, int p, __half v) {
    const int off = (r >> 3) * 1024 + (r & 7) * 128 + (((p >> 3) ^ (r & 7)) << 4) + (p & 7) * 2;
    *reinterpret_cast<__half*>(tile + off) = v;
}

__device__ __forceinline__ void tc_geom(const float4 P, float& ct, float2& z) {
    const float r = sqrtf(fmaf(P.z, P.z, fmaf(P.x, P.x, P.y * P.y)));
    ct = 1.f;
    z = make_float2(0.f, 0.f);
    if (r > 0.f) {
        const float ir = 1.f / r;
        ct = P.z * ir;
        z = make_float2(-P.x * ir, P.y * ir);
    }
}

// Octet of a step of the unit's sequence and the step within it.
__device__ __forceinline__ void tc_decode(int LM, int gs, int& o, int& d) {
    const int O = LM / 8 + 1;
    o = 0;
    while (o + 1 < O && tc_octet_first(LM, o + 1) <= gs) ++o;
    d = gs - tc_octet_first(LM, o);
}

// FP16 pair (x0 in the low half: the lower K index) as one register.
__device__ __forceinline__ uint32_t h2u(float x0, float x1) {
    const __half2 h = __floats2half2_rn(x0, x1);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ void hm_moments_tc(const float4* __restrict__ pts, const int4* __restrict__ units, int n_units, int K,
                              float delta, const int* __restrict__ lmb, const float2* __restrict__ cr,
                              const float* __restrict__ nmm, float2* __restrict__ MP, int64_t local) {
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    unsigned char* sm = tc_smem_raw + ((1024u - (smem_u32(tc_smem_raw) & 1023u)) & 1023u);
    unsigned char* sB = sm;
    float4* sP = reinterpret_cast<float4*>(sm + kTcOffP);
    float2* sZ8 = reinterpret_cast<float2*>(sm + kTcOffZ8);  // [o][64]
    float2* sZg = reinterpret_cast<float2*>(sm + kTcOffZg);  // [g][64]
    float* sAcc = reinterpret_cast<float*>(sm + kTcOffAcc);  // [tile][row][n]
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kTcOffBar);
    uint64_t* full = bars;
    uint64_t* empty = bars + 2;
    uint64_t* done = bars + 4;
    uint64_t* drained = bars + 4 + kTcTiles;
    volatile uint32_t* s_taddr = reinterpret_cast<volatile uint32_t*>(bars + kTcBars);
    volatile int* s_abort = reinterpret_cast<volatile int*>(bars + kTcBars) + 1;
    unsigned int* s_wmax = reinterpret_cast<unsigned int*>(bars + kTcBars + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // ---- the CTA's unit (the last whose first CTA <= local) and part ----
    int lo = 0, hi = n_units - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (units[mid].w <= local) lo = mid;
        else hi = mid - 1;
    }
    const int4 un = units[lo];
    const int LM = lmb[un.z];
    const int S = tc_steps(LM), P = tc_parts(LM), W = 4 * P;
    const int part = (int)(local - un.w);
    if (part < 0 || part >= P || un.y > kTcUnit) return;  // (uniform over the CTA)
    const int T = ((S + W - 1) / W + 1) / 2;  // tiles per chunk, every slot of the unit
    const int nch = (un.y + kTcChunk - 1) / kTcChunk;
    const int total = nch * T;

    if (tid == 0) {
        for (int k = 0; k < 2; ++k) {
            mbar_init(&full[k], 32 * kTcProducers);
            mbar_init(&empty[k], 1);
        }
        for (int k = 0; k < kTcTiles; ++k) {
            mbar_init(&done[k], 1);
            mbar_init(&drained[k], 32 * kTcDrainers);
        }
        *s_abort = 0;
        *s_wmax = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == kTcMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32((const void*)s_taddr)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int j = tid; j < kTcUnit; j += kTcThreads) sP[j] = j < un.y ? pts[un.x + j] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int e = tid; e < (int)(kTcOffP / 16); e += kTcThreads) reinterpret_cast<uint4*>(sB)[e] = make_uint4(0, 0, 0, 0);
    for (int e = tid; e < T * 128 * kNodes; e += kTcThreads) sAcc[e] = 0.f;
    __syncthreads();
    for (int j = tid; j < un.y; j += kTcThreads) atomicMax(s_wmax, __float_as_uint(fabsf(sP[j].w)));
    __syncthreads();
    int wexp = 0;
    frexpf(__uint_as_float(*s_wmax), &wexp);  // max |w| < 2^wexp
    const float wsc = ldexpf(1.f, kTcWeightExp - wexp), wback = ldexpf(1.f, wexp - kTcWeightExp - 11);
    {
        const float rb = (un.z + 0.5f) * delta, ih = 2.f / delta;
        for (int j = tid; j < un.y; j += kTcThreads) {
            const float4 Pt = sP[j];
            const float r = sqrtf(fmaf(Pt.z, Pt.z, fmaf(Pt.x, Pt.x, Pt.y * Pt.y)));
            const float u = (r - rb) * ih;
            unsigned char* tile = sB + (j / kTcChunk) * 2048;
            const int p = j % kTcChunk;
            float wv = Pt.w;  // w u^n, as hm_moments forms it, then scaled by 2^(14 - wexp)
            for (int n = 0; n < kNodes; ++n) {
                const float v = wv * wsc;
                const __half h = __float2half_rn(v);
                tc_put_weight(tile, n, p, h);
                tc_put_weight(tile, 6 + n, p, __float2half_rn(v - __half2float(h)));
                wv *= u;
            }
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the weights are read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *s_taddr;

    if (warp == kTcMmaWarp) {
        // ---- MMA issue: one thread ----
        if (lane == 0) {
            int issued = -1;
            for (int t = 0; t < total; ++t) {
                if (*s_abort) break;
                const int s = t & 1;
                const int c = t / T, tau = t - c * T;
                // the slot's basis values are in, and the tile's last sums were drained
                if (!mbar_wait(&full[s], (uint32_t)((t >> 1) & 1)) ||
                    (c > 0 && !mbar_wait(&drained[tau], (uint32_t)((c - 1) & 1)))) {
                    *s_abort = 1;
                    atomicOr(&g_tc_fault, 1u);
                    break;
                }
                tc_fence_after();
                const uint32_t d = tbase + kTcAcc0 + 16u * (uint32_t)tau;
                const uint32_t a = tbase + 64u * (uint32_t)s;
                const uint64_t bd = sw128_desc(smem_u32(sB + c * 2048));
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    mma_f16_ts(d, a + 8u * k, bd + 2u * k, kTcIdesc, k > 0 ? 1u : 0u);
                    mma_f16_ts(d, a + 32u + 8u * k, bd + 2u * k, kTcIdesc, 1u);
                }
                mma_commit(&empty[s]);
                mma_commit(&done[tau]);
                issued = t;
            }
            // the last commit covers every MMA this thread issued
            if (issued >= 0 && !mbar_wait(&empty[issued & 1], (uint32_t)((issued >> 1) & 1)))
                atomicOr(&g_tc_fault, 2u);
        }
        __syncwarp();
    } else if (warp > kTcMmaWarp) {
        // ---- drains: tile tau of chunk c into the FP32 sums, then free it ----
        const int qd = warp & 3;  // the lane quarter this warp may read
        for (int t = 0; t < total; ++t) {
            const int c = t / T, tau = t - c * T;
            if (!__all_sync(0xffffffffu, mbar_wait(&done[tau], (uint32_t)(c & 1)))) {
                *s_abort = 1;
                atomicOr(&g_tc_fault, 16u);
                break;
            }
            tc_fence_after();
            uint32_t v[16];
            tmem_ld_32x32b_x16(tbase + ((uint32_t)(32 * qd) << 16) + kTcAcc0 + 16u * (uint32_t)tau, v);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float* acc = sAcc + ((size_t)tau * 128 + 32 * qd + lane) * kNodes;
#pragma unroll
            for (int n = 0; n < kNodes; ++n) acc[n] += __uint_as_float(v[n]) + __uint_as_float(v[6 + n]);
            tc_fence_before();
            mbar_arrive(&drained[tau]);
        }
    } else {
        // ---- producers ----
        const int g = lane >> 2, t4 = lane & 3;
        const int sid = 4 * part + warp;
        const int g0 = (int)((int64_t)sid * S / W), g1 = (int)((int64_t)(sid + 1) * S / W);
        const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
        bool ok = true;
        // every producer warp passes the two named barriers of every chunk (an
        // abort only skips the chunk's tiles), so no warp waits on one that left
        for (int c = 0; c < nch; ++c) {
            // the chunk's power tables: z^g (g < 8) and z^(8o)
            producers_sync();
            if (tid < kTcChunk) {
                float ct;
                float2 z;
                tc_geom(sP[c * kTcChunk + tid], ct, z);
                float2 zp = make_float2(1.f, 0.f);
                for (int k = 0; k < 8; ++k) {
                    sZg[k * kTcChunk + tid] = zp;
                    zp = cmulf(zp, z);
                }
                float2 zo = make_float2(1.f, 0.f);
                const int O = LM / 8 + 1;
                for (int o = 0; o < O; ++o) {
                    sZ8[o * kTcChunk + tid] = zo;
                    zo = cmulf(zo, zp);
                }
            }
            producers_sync();
            if (__any_sync(0xffffffffu, !ok || *s_abort)) {  // (warp-uniform)
                ok = false;
                continue;
            }
            // the thread's 16 points: 16 rep + 4 t4 + i, as q = 4 rep + i
            f2x x2[16], q1[16], q2[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                float ct;
                float2 z;
                tc_geom(sP[c * kTcChunk + 16 * (q >> 2) + 4 * t4 + (q & 3)], ct, z);
                x2[q] = pk2(2.f * ct, 2.f * ct);
                q1[q] = q2[q] = 0ull;
            }
            int o = 0, d = 0;
            if (g0 < g1) tc_decode(LM, g0, o, d);
            int m = 8 * o + g;
            int Lo = LM + 1 - 8 * o;  // steps of octet o
            // one step of the recurrences at (o, d): q_l with l = m + d into q1
            auto advance = [&](float c_lm) {
                if (d == 0) {  // the octet's start: q_m = nmm[m] z^m, z^m = z^(8o) z^g
                    const float nm = m <= LM ? nmm[m] : 0.f;
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int pc = 16 * (q >> 2) + 4 * t4 + (q & 3);
                        const float2 zm = cmulf(sZ8[o * kTcChunk + pc], sZg[g * kTcChunk + pc]);
                        q2[q] = 0ull;
                        q1[q] = pk2(nm * zm.x, nm * zm.y);
                    }
                } else {
                    const f2x nc = pk2(-c_lm, -c_lm);
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const f2x v = fma2(x2[q], q1[q], mul2(nc, q2[q]));
                        q2[q] = q1[q];
                        q1[q] = v;
                    }
                }
            };
            // silent steps up to the slot's first
            {
                const int d0 = d;
                for (d = 0; d < d0; ++d) {
                    const int l = m + d;
                    const float c_lm = (d >= 2 && m <= LM && l <= LM) ? __ldg(&cr[l * (l + 1) / 2 + m].x) : 0.f;
                    advance(c_lm);
                }
            }
            int gs = g0;
            for (int tau = 0; tau < T; ++tau) {
                const int t = c * T + tau, s = t & 1;
                if (__any_sync(0xffffffffu, *s_abort != 0)) {
                    ok = false;
                    break;
                }
                // the warp decides together (the .sync.aligned stores below need every lane)
                const bool free = __all_sync(0xffffffffu, t < 2 || mbar_wait(&empty[s], (uint32_t)(((t >> 1) - 1) & 1)));
                if (!free) {
                    *s_abort = 1;
                    atomicOr(&g_tc_fault, 4u);
                    ok = false;
                    break;
                }
                tc_fence_after();
#pragma unroll 1
                for (int h = 0; h < 2; ++h, ++gs) {
                    uint32_t H[16], L[16];
                    if (gs < g1) {
                        if (d == Lo) {  // next octet
                            ++o;
                            d = 0;
                            m = 8 * o + g;
                            Lo = LM + 1 - 8 * o;
                        }
                        const int l = m + d;
                        const bool act = m <= LM && l <= LM;
                        float2 cv = make_float2(0.f, 0.f);
                        if (act) cv = __ldg(&cr[l * (l + 1) / 2 + m]);
                        advance(d >= 2 ? cv.x : 0.f);
                        // r_lm 2^11 (0 for rows past their last order)
                        const f2x r2 = pk2(cv.y * kTcBasisScale, cv.y * kTcBasisScale);
#pragma unroll
                        for (int rep = 0; rep < 4; ++rep) {
                            float hr[4], hi_[4], lr[4], li[4];
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const f2x v = mul2(q1[4 * rep + i], r2);
                                float vr, vi;
                                upk2(v, vr, vi);
                                const float ar = __uint_as_float(__float_as_uint(vr) & 0xffffe000u);
                                const float ai = __uint_as_float(__float_as_uint(vi) & 0xffffe000u);
                                float br, bi;
                                upk2(sub2(v, pk2(ar, ai)), br, bi);
                                hr[i] = ar;
                                hi_[i] = ai;
                                lr[i] = br;
                                li[i] = bi;
                            }
                            H[4 * rep + 0] = h2u(hr[0], hr[1]);
                            H[4 * rep + 1] = h2u(hr[2], hr[3]);
                            H[4 * rep + 2] = h2u(hi_[0], hi_[1]);
                            H[4 * rep + 3] = h2u(hi_[2], hi_[3]);
                            L[4 * rep + 0] = h2u(lr[0], lr[1]);
                            L[4 * rep + 1] = h2u(lr[2], lr[3]);
                            L[4 * rep + 2] = h2u(li[0], li[1]);
                            L[4 * rep + 3] = h2u(li[2], li[3]);
                        }
                        ++d;
                    } else {
#pragma unroll
                        for (int e = 0; e < 16; ++e) H[e] = L[e] = 0u;
                    }
                    const uint32_t ta = tbase + lane_base + ((uint32_t)(16 * h) << 16) + 64u * (uint32_t)s;
                    tmem_st_16x256b_x4(ta, H);
                    tmem_st_16x256b_x4(ta + 32u, L);
                }
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                tc_fence_before();
                mbar_arrive(&full[s]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp < kTcProducers && !*s_abort) {
        // ---- epilogue: row 32w + 16h + 8c + g of tile tau = (order of row g of
        // producer slot w's step 2 tau + h, component c) ----
        const int sid = 4 * part + warp;
        const int g0 = (int)((int64_t)sid * S / W), g1 = (int)((int64_t)(sid + 1) * S / W);
        const int h = lane >> 4, c = (lane >> 3) & 1, g = lane & 7;
        float* out = reinterpret_cast<float*>(MP);
        for (int tau = 0; tau < T; ++tau) {
            const int gs = g0 + 2 * tau + h;
            if (gs >= g1) continue;
            int o, d;
            tc_decode(LM, gs, o, d);
            const int m = 8 * o + g, l = m + d;
            if (m > LM || l > LM) continue;
            const int64_t k = (int64_t)l * (l + 1) / 2 + m;
            const float* acc = sAcc + ((size_t)tau * 128 + 32 * warp + lane) * kNodes;
#pragma unroll
            for (int n = 0; n < kNodes; ++n) out[(((int64_t)lo * kNodes + n) * K + k) * 2 + c] = acc[n] * wback;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kTcMmaWarp) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTcCols) : "memory");
    }
}

// ---------------------------------------------------------------------------
// tcgen05 issue calibration: one thread issues R = 32 MMAs of kind::f16,
// M = 128 (A in tensor memory, B in shared memory, zeros), N = 16 or 256, into
// one accumulator, and times (clock64) from the first issue to the commit's
// mbarrier completion: cycles[0] for N = 16, cycles[1] for N = 256, the best of
// 4 repetitions.  Bounded waits; status 1 when a wait ran out.
// ---------------------------------------------------------------------------
constexpr int kIssueProbeMmas = 32;
__global__ void __launch_bounds__(128, 1) tc_issue_probe_kernel(long long* cycles, int* status) {
    extern __shared__ __align__(1024) unsigned char pr_raw[];
    unsigned char* sm = pr_raw + ((1024u - (smem_u32(pr_raw) & 1023u)) & 1023u);
    unsigned char* sB = sm;  // 256 rows x 128 B of zeros
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 32768);
    volatile uint32_t* sta = reinterpret_cast<volatile uint32_t*>(sm + 32768 + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int e = tid; e < 32768 / 16; e += blockDim.x) reinterpret_cast<uint4*>(sB)[e] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32((const void*)sta)),
                     "r"(512u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tb = *sta;
    if (tid == 0) {
        const uint64_t bd = sw128_desc(smem_u32(sB));
        int phase = 0;
        for (int v = 0; v < 2; ++v) {
            const uint32_t n = v == 0 ? 16u : 256u;
            const uint32_t idesc = (1u << 4) | ((n >> 3) << 17) | ((128u >> 4) << 24);
            long long best = -1;
            for (int rep = 0; rep < 4; ++rep) {
                const long long t0 = clock64();
                for (int r = 0; r < kIssueProbeMmas; ++r)
                    mma_f16_ts(tb + 256u, tb + 8u * (uint32_t)(r & 3), bd, idesc, r > 0 ? 1u : 0u);
                mma_commit(bar);
                if (!mbar_wait(bar, (uint32_t)(phase & 1))) *status = 1;
                ++phase;
                const long long dt = clock64() - t0;
                if (best < 0 || dt < best) best = dt;
            }
            cycles[v] = best;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tb), "r"(512u) : "memory");
    }
}

// ---------------------------------------------------------------------------
// Pipe calibration (the denominators of the moments' roofline): independent
// chains per thread, long enough that launch costs vanish.
//   kind 0: scalar FP32 FMA, 8 chains        (2 flops per FMA)
//   kind 1: packed fma.rn.f32x2, 8 chains    (4 flops per instruction)
//   kind 2: mma.sync m16n8k8 TF32, 4 independent accumulators per warp
//           (2 x 16 x 8 x 8 = 2,048 flops per MMA)
//   kind 3: mma.sync m16n8k16 FP16 with FP32 accumulators, 4 independent
//           accumulators per warp (4,096 flops per MMA)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) pipe_probe_kernel(int kind, int iters, float* out) {
    float acc = 0.f;
    if (kind == 0) {
        float x[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = 1e-3f * (threadIdx.x + 1) + 0.1f * c;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int c = 0; c < 8; ++c) x[c] = fmaf(x[c], 0.999f, 1e-4f);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) acc += x[c];
    } else if (kind == 1) {
        f2x x[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = pk2(1e-3f * (threadIdx.x + 1) + 0.1f * c, 0.2f * c);
        const f2x m = pk2(0.999f, 0.998f), a = pk2(1e-4f, 2e-4f);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int c = 0; c < 8; ++c) x[c] = fma2(x[c], m, a);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            float u, v;
            upk2(x[c], u, v);
            acc += u + v;
        }
    } else if (kind == 2) {
        float d[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
        const uint32_t a[4] = {tf32_rna(1e-3f * threadIdx.x), tf32_rna(0.5f), tf32_rna(0.25f), tf32_rna(0.125f)};
        const uint32_t b0 = tf32_rna(1e-3f), b1 = tf32_rna(2e-3f);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int j = 0; j < 4; ++j) mma_tf32(d[j], a, b0, b1);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) acc += d[j][0] + d[j][1] + d[j][2] + d[j][3];
    } else {
        float d[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
        const uint32_t a[4] = {h2pack(1e-3f * threadIdx.x, 0.5f), h2pack(0.25f, 0.125f), h2pack(0.5f, 0.25f),
                               h2pack(0.125f, 1e-3f)};
        const uint32_t b0 = h2pack(1e-3f, 2e-3f), b1 = h2pack(3e-3f, 4e-3f);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int j = 0; j < 4; ++j) mma_f16(d[j], a, b0, b1);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) acc += d[j][0] + d[j][1] + d[j][2] + d[j][3];
    }
    if (acc == 12345.678f) out[0] = acc;  // keeps the chains live; never true for these inputs
}

// ---------------------------------------------------------------------------
// Solvent boxes to voxels, binned by radius with a stable counting sort:
// vx_expand (voxel v of box b: centre, weight; its bin; per-block histograms),
// vx_bins (per bin: the total and its blocks' offsets), vx_scatter (the rank of
// a voxel among the earlier voxels of its block and bin, by warp match and the
// per-warp counts).  The order within a bin is the voxel order: deterministic.
// boxes: float4 pairs {cx, cy, cz, w} about the centre, {Lx, Ly, Lz, 0};
// vstart[b]: first voxel of box b (z fastest, then y, then x).
// ---------------------------------------------------------------------------
constexpr int kBinThreads = 256;
constexpr int kMaxBins = 1024;

__global__ void __launch_bounds__(kBinThreads) vx_expand(const float4* __restrict__ boxes,
                                                         const int64_t* __restrict__ vstart, int64_t nb, int64_t nv,
                                                         float vs, float delta, int nbins, float4* __restrict__ vox,
                                                         int* __restrict__ vbin, int* __restrict__ hist, int nblk) {
    __shared__ int sh[kMaxBins];
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) sh[b] = 0;
    __syncthreads();
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nv) {
        int64_t lo = 0, hi = nb - 1;  // the last box with vstart <= v
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (vstart[mid] <= v) lo = mid;
            else hi = mid - 1;
        }
        const float4 c = boxes[2 * lo], L = boxes[2 * lo + 1];
        const int ny = __float2int_rn(L.y / vs), nz = __float2int_rn(L.z / vs);
        const int64_t local = v - vstart[lo];
        const int iz = (int)(local % nz);
        const int64_t rest = local / nz;
        const int iy = (int)(rest % ny), ix = (int)(rest / ny);
        const float4 p = make_float4(c.x + ((ix + 0.5f) * vs - 0.5f * L.x), c.y + ((iy + 0.5f) * vs - 0.5f * L.y),
                                     c.z + ((iz + 0.5f) * vs - 0.5f * L.z), c.w);
        vox[v] = p;
        const float r = sqrtf(fmaf(p.x, p.x, fmaf(p.y, p.y, p.z * p.z)));
        const int b = min(nbins - 1, (int)(r / delta));
        vbin[v] = b;
        atomicAdd(&sh[b], 1);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) hist[(int64_t)b * nblk + blockIdx.x] = sh[b];
}

// Block-wide exclusive scan of one int64 per thread; returns the thread's
// prefix, *total the block's sum.
__device__ __forceinline__ int64_t block_scan_excl(int64_t v, int64_t* total) {
    __shared__ int64_t ws[32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    int64_t before = 0, all = 0;
    for (int k = 0; k < nw; ++k) {
        if (k < w) before += ws[k];
        all += ws[k];
    }
    __syncthreads();
    *total = all;
    return before + x - v;
}

// The leaf's solvent boxes (raw D+ records {cx, cy, cz, w, Lx, Ly, Lz, -}) about
// the centre c: the float4 pair {centre - c, w}, {L, 0}; each box's voxel
// count (its edges over the voxel step, rounded as vx_expand rounds them); the
// largest squared distance of a box corner from c and of a voxel centre (the
// corner of the box shrunk by half a voxel), rounded up to FP32, and the total
// voxel count, reduced into scal = {corner r2 bits, total, centre r2 bits}.
__global__ void __launch_bounds__(kBinThreads) vx_prepare(const float* __restrict__ raw, int64_t nb, double cx,
                                                          double cy, double cz, float vs, float4* __restrict__ boxes,
                                                          int64_t* __restrict__ counts,
                                                          unsigned long long* __restrict__ scal) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float q = 0.f, qv = 0.f;
    int64_t n = 0;
    if (b < nb) {
        const float* r = raw + 8 * b;
        const double c[3] = {cx, cy, cz};
        double e2 = 0.0, v2 = 0.0;
        for (int k = 0; k < 3; ++k) {
            const double d = fabs((double)r[k] - c[k]);
            const double e = d + 0.5 * (double)r[4 + k];
            const double v = d + 0.5 * fmax((double)r[4 + k] - (double)vs, 0.0);
            e2 += e * e;
            v2 += v * v;
        }
        q = __double2float_ru(e2);
        qv = __double2float_ru(v2);
        boxes[2 * b] = make_float4((float)((double)r[0] - cx), (float)((double)r[1] - cy), (float)((double)r[2] - cz),
                                   r[3]);
        boxes[2 * b + 1] = make_float4(r[4], r[5], r[6], 0.f);
        n = (int64_t)__float2int_rn(r[4] / vs) * __float2int_rn(r[5] / vs) * __float2int_rn(r[6] / vs);
        counts[b] = n;
    }
    // block reduction, then one atomic each
    unsigned qb = __float_as_uint(q), qvb = __float_as_uint(qv);  // >= 0: the bits order as the values
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        qb = max(qb, __shfl_down_sync(0xffffffffu, qb, o));
        qvb = max(qvb, __shfl_down_sync(0xffffffffu, qvb, o));
        n += __shfl_down_sync(0xffffffffu, n, o);
    }
    __shared__ unsigned sq[kBinThreads / 32], sqv[kBinThreads / 32];
    __shared__ int64_t sn[kBinThreads / 32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sq[w] = qb;
        sqv[w] = qvb;
        sn[w] = n;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned qm = 0, qvm = 0;
        int64_t nt = 0;
        for (int k = 0; k < kBinThreads / 32; ++k) {
            qm = max(qm, sq[k]);
            qvm = max(qvm, sqv[k]);
            nt += sn[k];
        }
        atomicMax(scal, (unsigned long long)qm);
        atomicAdd(scal + 1, (unsigned long long)nt);
        atomicMax(scal + 2, (unsigned long long)qvm);
    }
}

// vstart = exclusive prefix of the box voxel counts, over runs of
// kVstartRun boxes: vx_run_sums gives each run's total; vx_vstart adds the
// totals of the earlier runs and scans its own (kBinThreads threads, a
// contiguous stretch of the run per thread).
constexpr int kVstartRun = kVoxelScanRun;
static_assert(kVstartRun % kBinThreads == 0, "a scan run is whole stretches of the block's threads");

__global__ void __launch_bounds__(kBinThreads) vx_run_sums(const int64_t* __restrict__ counts, int64_t nb,
                                                           int64_t* __restrict__ sums) {
    const int64_t r0 = (int64_t)blockIdx.x * kVstartRun;
    int64_t v = 0;
    for (int k = threadIdx.x; k < kVstartRun; k += blockDim.x)
        if (r0 + k < nb) v += counts[r0 + k];
    int64_t all;
    block_scan_excl(v, &all);
    if (threadIdx.x == 0) sums[blockIdx.x] = all;
}

__global__ void __launch_bounds__(kBinThreads) vx_vstart(const int64_t* __restrict__ counts, int64_t nb,
                                                         const int64_t* __restrict__ sums,
                                                         int64_t* __restrict__ vstart) {
    int64_t before = 0;
    for (int k = threadIdx.x; k < (int)blockIdx.x; k += blockDim.x) before += sums[k];
    int64_t start;
    block_scan_excl(before, &start);
    const int64_t r0 = (int64_t)blockIdx.x * kVstartRun;
    const int per = kVstartRun / kBinThreads;
    const int64_t b0 = min(nb, r0 + (int64_t)threadIdx.x * per), b1 = min(nb, b0 + per);
    int64_t mine = 0;
    for (int64_t b = b0; b < b1; ++b) mine += counts[b];
    int64_t dummy;
    int64_t run = start + block_scan_excl(mine, &dummy);
    for (int64_t b = b0; b < b1; ++b) {
        vstart[b] = run;
        run += counts[b];
    }
}

// block per bin: its total over the expand blocks
__global__ void __launch_bounds__(kBinThreads) vx_totals(const int* __restrict__ hist, int nbins, int nblk,
                                                         int64_t* __restrict__ total) {
    const int b = blockIdx.x;
    int64_t v = 0;
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) v += hist[(int64_t)b * nblk + k];
    int64_t all;
    block_scan_excl(v, &all);
    if (threadIdx.x == 0) total[b] = all;
}

// block per bin: off[b][blk] = start of bin b + the counts of its earlier
// blocks (a contiguous run of blocks per thread, then a block scan)
__global__ void __launch_bounds__(kBinThreads) vx_offsets(const int* __restrict__ hist,
                                                          const int64_t* __restrict__ total, int nbins, int nblk,
                                                          int64_t* __restrict__ off) {
    const int b = blockIdx.x;
    int64_t before = 0;
    for (int c = threadIdx.x; c < b; c += blockDim.x) before += total[c];
    int64_t start;
    block_scan_excl(before, &start);
    const int per = (nblk + kBinThreads - 1) / kBinThreads;
    const int k0 = min(nblk, (int)threadIdx.x * per), k1 = min(nblk, k0 + per);
    const int* hb = hist + (int64_t)b * nblk;
    int64_t mine = 0;
    for (int k = k0; k < k1; ++k) mine += hb[k];
    int64_t dummy;
    int64_t run = start + block_scan_excl(mine, &dummy);
    for (int k = k0; k < k1; ++k) {
        off[(int64_t)b * nblk + k] = run;
        run += hb[k];
    }
}

__global__ void __launch_bounds__(kBinThreads) vx_scatter(const float4* __restrict__ vox, const int* __restrict__ vbin,
                                                          int64_t nv, int nbins, int nblk,
                                                          const int64_t* __restrict__ off, float4* __restrict__ out) {
    __shared__ int wc[kBinThreads / 32][kMaxBins];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int e = threadIdx.x; e < (kBinThreads / 32) * nbins; e += blockDim.x) wc[e / nbins][e % nbins] = 0;
    __syncthreads();
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = v < nv;
    const int b = valid ? vbin[v] : -1 - lane;  // invalid lanes form groups of one
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wc[w][b] = __popc(peers);
    __syncthreads();
    if (valid) {
        int pre = 0;
        for (int k = 0; k < w; ++k) pre += wc[k][b];
        out[off[(int64_t)b * nblk + blockIdx.x] + pre + rank] = vox[v];
    }
}

// s += x with the rounding error of every addition carried in c (Knuth's
// TwoSum): a compensated FP32 sum, about as accurate as an FP64 one.
__device__ __forceinline__ void sum2(float& s, float& c, float x) {
    const float t = s + x;
    const float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
}

// hm_groups: M[g][n][k] = sum of MP over the units [gu[g], gu[g+1]) of group g,
// compensated.
__device__ void hm_groups(const float2* __restrict__ MP, const int* __restrict__ gu, const int2* __restrict__ groups,
                          const int* __restrict__ lmb, int G, int K, float2* __restrict__ M, int64_t e) {
    const int64_t per = (int64_t)kNodes * K;
    if (e >= (int64_t)G * per) return;
    const int g = (int)(e / per);
    const int64_t r = e % per;
    const int lb = lmb[groups[g].x];
    if ((int)(r % K) >= (lb + 1) * (lb + 2) / 2) {  // orders the group's bin does not carry
        M[e] = make_float2(0.f, 0.f);
        return;
    }
    float re = 0.f, rc = 0.f, im = 0.f, ic = 0.f;
    for (int u = gu[g]; u < gu[g + 1]; ++u) {
        const float2 v = MP[(int64_t)u * per + r];
        sum2(re, rc, v.x);
        sum2(im, ic, v.y);
    }
    M[e] = make_float2(re + rc, im + ic);
}

// ---------------------------------------------------------------------------
// hm_contract: block (k slice of 32, tile of 8 shells), four warps; lane k,
// warp w sums the groups [w G / 4, (w + 1) G / 4) (compensated), and the four
// partial sums are combined in a fixed order with the same compensation.
// groups[g] = {bin, ion (< 0: factor 1)}; C[i][k] = sum_g F sum_n T M.
// ---------------------------------------------------------------------------
constexpr int kContractShells = 8;
constexpr int kContractK = 32;
constexpr int kContractWarps = 4;

__device__ void hm_contract(const float2* __restrict__ M, const int2* __restrict__ groups, int G,
                            const float* __restrict__ T, int nbins, int LM, int K, int Lp, const int* __restrict__ lmax,
                            const int* __restrict__ lmb, const float* __restrict__ aff, float2* __restrict__ C, int bx,
                            int by) {
    __shared__ float4 part[kContractWarps][kContractShells][kContractK];  // {s_re, c_re, s_im, c_im}
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int k = bx * kContractK + lane;
    const int i0 = 1 + by * kContractShells;
    const bool kok = k < K;
    const int l = kok ? l_of(k) : 0;
    float cr[kContractShells], ci[kContractShells], er[kContractShells], ei[kContractShells];
#pragma unroll
    for (int a = 0; a < kContractShells; ++a) cr[a] = ci[a] = er[a] = ei[a] = 0.f;
    const int g0 = (int)((int64_t)G * w / kContractWarps), g1 = (int)((int64_t)G * (w + 1) / kContractWarps);
    if (kok) {
        for (int g = g0; g < g1; ++g) {
            const int2 gb = groups[g];
            if (l > lmb[gb.x]) continue;  // zero moments: the bin needs no order l
            float2 mv[kNodes];
#pragma unroll
            for (int n = 0; n < kNodes; ++n) mv[n] = M[((int64_t)g * kNodes + n) * K + k];
#pragma unroll
            for (int a = 0; a < kContractShells; ++a) {
                const int i = i0 + a;
                if (i > Lp || lmax[i] < l) continue;
                const float4* t4 = reinterpret_cast<const float4*>(T + (((int64_t)i * nbins + gb.x) * (LM + 1) + l) * 8);
                const float4 ta = t4[0], tb = t4[1];
                const float t[kNodes] = {ta.x, ta.y, ta.z, ta.w, tb.x, tb.y};
                float sr = 0.f, si = 0.f;
#pragma unroll
                for (int n = 0; n < kNodes; ++n) {
                    sr = fmaf(t[n], mv[n].x, sr);
                    si = fmaf(t[n], mv[n].y, si);
                }
                const float f = gb.y < 0 ? 1.f : aff[(int64_t)gb.y * (Lp + 1) + i];
                sum2(cr[a], er[a], __fmul_rn(f, sr));
                sum2(ci[a], ei[a], __fmul_rn(f, si));
            }
        }
    }
#pragma unroll
    for (int a = 0; a < kContractShells; ++a) part[w][a][lane] = make_float4(cr[a], er[a], ci[a], ei[a]);
    __syncthreads();
    // warp a' < kContractShells / ... : thread (shell a, lane) combines the four warps
    for (int e = threadIdx.x; e < kContractShells * kContractK; e += blockDim.x) {
        const int a = e / kContractK, kl = e % kContractK;
        const int i = i0 + a, kk = bx * kContractK + kl;
        if (i > Lp || kk >= K) continue;
        float sr = 0.f, srr = 0.f, si = 0.f, sii = 0.f;
#pragma unroll
        for (int ww = 0; ww < kContractWarps; ++ww) {
            const float4 p = part[ww][a][kl];
            sum2(sr, srr, p.x);
            srr += p.y;
            sum2(si, sii, p.z);
            sii += p.w;
        }
        C[(int64_t)i * K + kk] = make_float2(sr + srr, si + sii);
    }
}

__device__ __forceinline__ float sinc_h(float h) {
    const float h2 = h * h;
    if (h2 < 0.25f) return fmaf(h2, fmaf(h2, fmaf(h2, -1.f / 5040.f, 1.f / 120.f), -1.f / 6.f), 1.f);
    return __fdividef(__sinf(h), h);
}

// ---------------------------------------------------------------------------
// hm_synth: block (row group, shell i): up to kSynthRows theta rows t <= 3i/2
// of one shell.  A row's 6i cells are F(p) = sum_{|m| <= l_i} G_m w^{mp},
// w = e^{2 pi i/6i}, with G_m = 4 pi sum_l i^l P_lm C_lm and
// G_-m = 4 pi sum_l i^l P_lm conj(C_lm) (m > 0).
//   G stage: a warp takes four orders m x eight rows (lane = m, row), runs the
//   Legendre recurrence of its (m, row) in registers and sums against the
//   shell's C_lm (the eight lanes of an order read one address, a warp one
//   32-byte sector); the quartets are dealt to the warps from both ends.
//   Cell stage: writing p = s i + j (sextant s < 6, column j < i),
//     F(s i + j) = sum_{r < 6} e^{2 pi i r s / 6} D_r(j),
//     D_r(j) = sum_{m = r mod 6} G_m w^{mj},
//   so a thread per (row, column j) sums the G_m once into six residue
//   classes (each by Horner's rule in z = w^{6j}: D_r(j) = w^{m_r j}
//   sum_k G_{m_r + 6k} z^k, m_r the class's lowest order) and finishes its six
//   cells with a 6-point DFT; as many rows run at
//   once as 256 threads have columns for.  Then the voxel form factor, the
//   centring phase (double-float), and the rows' phi-spline derivatives
//   (row_spline, as the spline pass computes them) written with the values;
//   the Friedel mirror row gets the conjugates of both.
// Dynamic shared memory: G (atoms, voxels) per row over m in [m0, m0 + nG)
// with zero padding (m0 = -6 ceil(l_i/6)), the 6i roots of unity, the values
// of the rows in flight (6 max(256, 2 Lp) cells).
// ---------------------------------------------------------------------------
constexpr int kSynthThreads = 256;
constexpr int kSynthRows = 8;

__device__ __forceinline__ int synth_pad(int li) { return 6 * ((li + 5) / 6) + 6 * ((li + 6) / 6); }

__device__ __forceinline__ float2 i_pow_times(int l, float2 c) {  // i^l c
    switch (l & 3) {
        case 0: return c;
        case 1: return make_float2(-c.y, c.x);
        case 2: return make_float2(-c.x, -c.y);
        default: return make_float2(c.y, -c.x);
    }
}

// x = hi + lo (the FP32 pair nearest the FP64 value)
__device__ __forceinline__ float2 split_ff(double x) {
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

// X[s] = sum_{c < 6} D[c] e^{2 pi i c s / 6}: E = DFT3 of the even classes,
// O = DFT3 of the odd ones (e^{2 pi i / 3} steps), X[s] = E[s mod 3] +
// e^{i pi s / 3} O[s mod 3], X[s + 3] = E[s] - e^{i pi s / 3} O[s].
__device__ __forceinline__ void dft3(float2 a, float2 b, float2 c, float2& x0, float2& x1, float2& x2) {
    constexpr float kS3 = 0.86602540378443865f;  // sin(pi/3)
    const float2 t1 = make_float2(b.x + c.x, b.y + c.y);
    const float2 t2 = make_float2(fmaf(-0.5f, t1.x, a.x), fmaf(-0.5f, t1.y, a.y));
    const float2 t3 = make_float2(-kS3 * (b.y - c.y), kS3 * (b.x - c.x));  // i sin(pi/3) (b - c)
    x0 = make_float2(a.x + t1.x, a.y + t1.y);
    x1 = make_float2(t2.x + t3.x, t2.y + t3.y);
    x2 = make_float2(t2.x - t3.x, t2.y - t3.y);
}
__device__ __forceinline__ void dft6(const float2 (&D)[6], float2 (&X)[6]) {
    constexpr float kS3 = 0.86602540378443865f;
    float2 E[3], O[3];
    dft3(D[0], D[2], D[4], E[0], E[1], E[2]);
    dft3(D[1], D[3], D[5], O[0], O[1], O[2]);
    // twiddles e^{i pi s / 3}: 1, (1/2, sin(pi/3)), (-1/2, sin(pi/3))
    const float2 o1 = make_float2(0.5f * O[1].x - kS3 * O[1].y, kS3 * O[1].x + 0.5f * O[1].y);
    const float2 o2 = make_float2(-0.5f * O[2].x - kS3 * O[2].y, kS3 * O[2].x - 0.5f * O[2].y);
    X[0] = make_float2(E[0].x + O[0].x, E[0].y + O[0].y);
    X[3] = make_float2(E[0].x - O[0].x, E[0].y - O[0].y);
    X[1] = make_float2(E[1].x + o1.x, E[1].y + o1.y);
    X[4] = make_float2(E[1].x - o1.x, E[1].y - o1.y);
    X[2] = make_float2(E[2].x + o2.x, E[2].y + o2.y);
    X[5] = make_float2(E[2].x - o2.x, E[2].y - o2.y);
}

__device__ void hm_synth(int Lp, const float2* __restrict__ Ca,
                                                          const float2* __restrict__ Cv, int K,
                                                          const int* __restrict__ lmax, const float2* __restrict__ ab,
                                                          const float* __restrict__ nmm, double step, float vox_s,
                                                          double cx, double cy, double cz, int use_center, float scale,
                                                          double origin, float4* __restrict__ grid, int bx, int by) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ float2 sRow[kSynthRows][4];  // per row: {st, ct}, A, B, Z (double-float)
    const int i = by + 1;
    const int h = 3 * i, nph = 6 * i;
    const int rows_i = h / 2 + 1;  // rows t = 0 .. floor(3i/2)
    const int t0 = bx * kSynthRows;
    if (t0 >= rows_i) return;
    const int nr = min(kSynthRows, rows_i - t0);
    const int li = lmax[i];
    const int nG = synth_pad(li);
    const int m0p = -6 * ((li + 5) / 6);
    const bool vox = Cv != nullptr;
    // G per row: [set (atoms, voxels)][component (re, im)][nG] floats, so that
    // two neighbouring orders of one component load as one f32x2 pair
    float* sG = reinterpret_cast<float*>(smem);
    float2* sW = reinterpret_cast<float2*>(sG + (size_t)kSynthRows * 4 * nG);  // [6i]
    float2* sF = sW + nph;                              // [6 max(256, 2 Lp)]
    const int tid = threadIdx.x;
    for (int n = tid; n < nph; n += blockDim.x) {
        float sw, cw;
        sincospif(2.f * (float)n / (float)nph, &sw, &cw);
        sW[n] = make_float2(cw, sw);
    }
    for (int e = tid; e < nr * 4 * nG; e += blockDim.x) {  // the padding beyond |m| <= l_i
        const int m = m0p + e % nG;
        if (m > li || m < -li) sG[e] = 0.f;
    }
    const float qI = (float)((double)i * step);
    if (tid < nr) {
        const int t = t0 + tid;
        float st, ct;
        sincospif((float)t / (float)h, &st, &ct);
        sRow[tid][0] = make_float2(st, ct);
        // centring phase q.c / 2 pi = A cos(phi) + B sin(phi) + Z per cell, the
        // row constants in FP64, held as FP32 pairs
        const double inv2pi = 0.15915494309189533577;
        double sd, cd;
        sincospi((double)t / (double)h, &sd, &cd);
        const double qd = (double)i * step;
        sRow[tid][1] = split_ff(qd * sd * cx * inv2pi);
        sRow[tid][2] = split_ff(qd * sd * cy * inv2pi);
        sRow[tid][3] = split_ff(qd * cd * cz * inv2pi);
    }
    __syncthreads();
    // ---- G stage ----
    {
        const int warp = tid >> 5, lane = tid & 31;
        const int mq = lane >> 3, r = lane & 7;  // order 4q + mq, row t0 + r
        const int nq = (li + 4) / 4;
        const float2 sc = sRow[min(r, nr - 1)][0];
        const float st = sc.x, ct = sc.y;
        const float2* Cai = Ca + (int64_t)i * K;
        const float2* Cvi = vox ? Cv + (int64_t)i * K : nullptr;
        for (int o = warp; o < nq; o += kSynthThreads / 32) {
            const int q = (o & 1) ? nq - 1 - (o >> 1) : (o >> 1);  // 0, nq-1, 1, nq-2, ...
            const int m = 4 * q + mq;
            const bool ok = m <= li && r < nr;
            // Pbar_mm = nmm[m] (-sin theta)^m by binary powering
            float pmm = ok ? nmm[m] : 0.f, base = -st;
            for (int e = ok ? m : 0; e > 0; e >>= 1) {
                if (e & 1) pmm *= base;
                base *= base;
            }
            float p1 = 0.f, p2 = 0.f;
            float br = 0.f, bi = 0.f, pr = 0.f, pi_ = 0.f, vr = 0.f, vi = 0.f, qr = 0.f, qi = 0.f;
            int k = ok ? m * (m + 1) / 2 + m : 0;  // k(l, m) from l = m
            for (int l = 4 * q; l <= li; ++l) {
                float p = 0.f;
                if (ok && l >= m) {
                    if (l == m) {
                        p = pmm;
                    } else {
                        const float2 c = __ldg(&ab[k]);
                        p = c.x * fmaf(ct, p1, -c.y * p2);
                    }
                    const float2 cA = __ldg(&Cai[k]);
                    const float2 a = i_pow_times(l, cA), e = i_pow_times(l, make_float2(cA.x, -cA.y));
                    br = fmaf(p, a.x, br);
                    bi = fmaf(p, a.y, bi);
                    pr = fmaf(p, e.x, pr);
                    pi_ = fmaf(p, e.y, pi_);
                    if (vox) {
                        const float2 cV = __ldg(&Cvi[k]);
                        const float2 av = i_pow_times(l, cV), ev = i_pow_times(l, make_float2(cV.x, -cV.y));
                        vr = fmaf(p, av.x, vr);
                        vi = fmaf(p, av.y, vi);
                        qr = fmaf(p, ev.x, qr);
                        qi = fmaf(p, ev.y, qi);
                    }
                    p2 = p1;
                    p1 = p;
                    k += l + 1;  // k(l + 1, m)
                }
            }
            if (ok) {
                float* g = sG + (size_t)r * 4 * nG;
                g[m - m0p] = kFourPi * br;
                g[nG + m - m0p] = kFourPi * bi;
                if (m > 0) {
                    g[-m - m0p] = kFourPi * pr;
                    g[nG - m - m0p] = kFourPi * pi_;
                }
                if (vox) {
                    g[2 * nG + m - m0p] = kFourPi * vr;
                    g[3 * nG + m - m0p] = kFourPi * vi;
                    if (m > 0) {
                        g[2 * nG - m - m0p] = kFourPi * qr;
                        g[3 * nG - m - m0p] = kFourPi * qi;
                    }
                }
            }
        }
    }
    __syncthreads();
    // ---- cell stage: rpp rows at a time ----
    const int64_t base = shell_base(i);
    // rows in flight: as many as 256 threads have columns for, and at least
    // two (so that a large shell keeps more than i of the 256 threads busy)
    const int rpp = min(nr, max(2, kSynthThreads / i));
    for (int r0 = 0; r0 < nr; r0 += rpp) {
        const int nrp = min(rpp, nr - r0);
        for (int it = tid; it < nrp * i; it += blockDim.x) {
            const int rr = it / i, j = it - rr * i;
            const int r = r0 + rr;
            const float* gx = sG + (size_t)r * 4 * nG;  // atoms re, im; voxels re, im
            float2 D[6], Dv[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) D[c] = Dv[c] = make_float2(0.f, 0.f);
            // D_c = w^{(m0 + c) j} sum_k G_{m0 + c + 6k} z^k with z = w^{6j}: Horner
            // over k (no twiddle lookups in the loop), then one twiddle per class.
            // Classes in pairs (c, c + 1) as f32x2: X = re, Y = im of both,
            //   X' = X z.x + (Y (-z.y) + G.re),  Y' = X z.y + (Y z.x + G.im)
            // (per lane the same FP32 FMAs as the complex Horner step).
            const float2 z = sW[6 * j];
            const f2x ZX = pk2(z.x, z.x), ZY = pk2(z.y, z.y), NZY = pk2(-z.y, -z.y);
            const int top = nG - 6;
            auto ld2 = [](const float* p) { return *reinterpret_cast<const f2x*>(p); };
            f2x XA[3], YA[3], XV[3], YV[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                XA[q] = ld2(gx + top + 2 * q);
                YA[q] = ld2(gx + nG + top + 2 * q);
                XV[q] = YV[q] = 0ull;
                if (vox) {
                    XV[q] = ld2(gx + 2 * nG + top + 2 * q);
                    YV[q] = ld2(gx + 3 * nG + top + 2 * q);
                }
            }
            for (int u = top - 6; u >= 0; u -= 6) {
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const f2x xa = XA[q], ya = YA[q];
                    XA[q] = fma2(xa, ZX, fma2(ya, NZY, ld2(gx + u + 2 * q)));
                    YA[q] = fma2(xa, ZY, fma2(ya, ZX, ld2(gx + nG + u + 2 * q)));
                    if (vox) {
                        const f2x xv = XV[q], yv = YV[q];
                        XV[q] = fma2(xv, ZX, fma2(yv, NZY, ld2(gx + 2 * nG + u + 2 * q)));
                        YV[q] = fma2(xv, ZY, fma2(yv, ZX, ld2(gx + 3 * nG + u + 2 * q)));
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                upk2(XA[q], D[2 * q].x, D[2 * q + 1].x);
                upk2(YA[q], D[2 * q].y, D[2 * q + 1].y);
                if (vox) {
                    upk2(XV[q], Dv[2 * q].x, Dv[2 * q + 1].x);
                    upk2(YV[q], Dv[2 * q].y, Dv[2 * q + 1].y);
                }
            }
            int idx = (int)(((int64_t)m0p * j) % nph);
            if (idx < 0) idx += nph;
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const float2 w = sW[idx];
                D[c] = make_float2(fmaf(D[c].x, w.x, -D[c].y * w.y), fmaf(D[c].x, w.y, D[c].y * w.x));
                if (vox) Dv[c] = make_float2(fmaf(Dv[c].x, w.x, -Dv[c].y * w.y), fmaf(Dv[c].x, w.y, Dv[c].y * w.x));
                idx += j;  // idx, j < 6i
                if (idx >= nph) idx -= nph;
            }
            const float st = sRow[r][0].x, ct = sRow[r][0].y;
            const float2 A2 = sRow[r][1], B2 = sRow[r][2], Z2 = sRow[r][3];
            // the six sextants X[sx] = sum_c D_c e^{2 pi i c sx / 6} as two 3-point
            // DFTs (even and odd classes) and one radix-2 step
            float2 X[6], Xv[6];
            dft6(D, X);
            if (vox) dft6(Dv, Xv);
            const float qz = qI * ct;
            const float sz = vox ? sinc_h(0.5f * qz * vox_s) : 0.f;  // the row's z factor
#pragma unroll
            for (int sx = 0; sx < 6; ++sx) {
                float ar = X[sx].x, ai = X[sx].y;
                const int p = sx * i + j;
                const float2 w = sW[p];  // (cos, sin) of the cell's phi = p pi / 3i
                const float cp = w.x, sp = w.y;
                const float qx = qI * st * cp, qy = qI * st * sp;
                if (vox) {
                    const float f = vox_s * sinc_h(0.5f * qx * vox_s) * vox_s * sinc_h(0.5f * qy * vox_s) * vox_s * sz;
                    ar = fmaf(f, Xv[sx].x, ar);
                    ai = fmaf(f, Xv[sx].y, ai);
                }
                float2 F = make_float2(ar * scale, ai * scale);
                if (use_center) {
                    // turns = A cp + B sp + Z in double-float (Dekker's two-product,
                    // Knuth's two-sum), reduced by its nearest integer
                    const float p1 = __fmul_rn(A2.x, cp), e1 = fmaf(A2.x, cp, -p1);
                    const float p2 = __fmul_rn(B2.x, sp), e2 = fmaf(B2.x, sp, -p2);
                    const float s1 = __fadd_rn(p1, p2);
                    const float b1 = __fsub_rn(s1, p1);
                    const float f1 = __fadd_rn(__fsub_rn(p1, __fsub_rn(s1, b1)), __fsub_rn(p2, b1));
                    const float s2 = __fadd_rn(s1, Z2.x);
                    const float b2 = __fsub_rn(s2, s1);
                    const float f2 = __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, b2)), __fsub_rn(Z2.x, b2));
                    const float lo = e1 + e2 + f1 + f2 + Z2.y + A2.y * cp + B2.y * sp;
                    const float rt = __fsub_rn(s2, rintf(s2)) + lo;
                    float s1n, c1n;
                    sincospif(2.f * rt, &s1n, &c1n);
                    F = make_float2(F.x * c1n - F.y * s1n, F.x * s1n + F.y * c1n);
                }
                sF[rr * nph + p] = F;
            }
        }
        __syncthreads();
        for (int it = tid; it < nrp * nph; it += blockDim.x) {
            const int rr = it / nph, p = it - rr * nph;
            const int t = t0 + r0 + rr;
            const float2* row = sF + rr * nph;
            const float2 F = row[p];
            float dr, di;
            row_spline<float, 14>(nph, p, [&](int k) { return row[k]; }, dr, di);
            grid[base + (int64_t)t * nph + p] = make_float4(F.x, F.y, dr, di);
            // Friedel: the antipode (3i - t, p + 3i) holds the conjugate (the
            // equator row is its own mirror and is written once per cell)
            if (2 * t != h) {
                const int pm = p < h ? p + h : p - h;
                grid[base + (int64_t)(h - t) * nph + pm] = make_float4(F.x, -F.y, dr, -di);
            }
        }
        __syncthreads();
    }
    if (i == 1 && t0 == 0 && tid == 0) grid[0] = make_float4((float)origin, 0.f, 0.f, 0.f);
}

// ---------------------------------------------------------------------------
// Batched launches over a job table (HarmJob): a block finds its job (or its
// job's point set) by a binary search over the first blocks, then runs the
// body above with its local block index: the radial nodes of every job; the
// moments of every (job, set); the radial fit, then the group sums, in one
// launch; the contraction of every (job, set) whose coefficient set the
// synthesis reads; the synthesis of every job.
// ---------------------------------------------------------------------------
constexpr int kNodesThreads = 128, kFitThreads = 256;

__device__ __forceinline__ int job_of(const HarmJob* __restrict__ J, int n, int64_t blk, int64_t HarmJob::*key) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (J[mid].*key <= blk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
// (job, set) 2j + k of a per-set launch: the last with its first block <= blk
__device__ __forceinline__ int set_of(const HarmJob* __restrict__ J, int n, int64_t blk, int64_t (HarmJob::*key)[2]) {
    int lo = 0, hi = 2 * n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((J[mid >> 1].*key)[mid & 1] <= blk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int synth_groups(int Lp) { return (3 * Lp / 2 + 1 + kSynthRows - 1) / kSynthRows; }

// The radial tables of one plan (launch_radial_tables).
__global__ void __launch_bounds__(kNodesThreads) hm_nodes_plan(RadialTableArgs a) {
    hm_nodes(a.Lp, a.nbins, a.LM, a.step, a.delta, a.lmax, a.nodes, a.Jn,
             (int64_t)blockIdx.x * kNodesThreads + threadIdx.x);
}
__global__ void __launch_bounds__(kFitThreads) hm_fit_plan(RadialTableArgs a) {
    hm_fit(a.Lp, a.nbins, a.LM, a.lmax, a.vinv, a.Jn, a.T, (int64_t)blockIdx.x * kFitThreads + threadIdx.x);
}

template <bool H>
__global__ void __launch_bounds__(32) hm_moments_jobs(const HarmJob* __restrict__ J, int n,
                                                      char* __restrict__ scratch) {
    const int64_t b = blockIdx.x;
    const int js = set_of(J, n, b, &HarmJob::b_mom);
    const HarmJob& h = J[js >> 1];
    const int k = js & 1;
    const int64_t local = b - h.b_mom[k];
    const int nu = h.n_units[k];
    hm_moments<H>(h.pts[k], h.units[k], h.K, (float)h.delta, h.lmb, h.cr, h.nmm,
                  reinterpret_cast<float2*>(scratch + h.s_MP[k]), (int)(local % nu), (int)(local / nu));
}

// The tensor-core moments of every (job, set): a set's CTAs are its units'
// parts (units[].w: the unit's first CTA in the set).
__global__ void __launch_bounds__(kTcThreads, 1) hm_moments_tc_jobs(const HarmJob* __restrict__ J, int n,
                                                                    char* __restrict__ scratch) {
    const int64_t b = blockIdx.x;
    const int js = set_of(J, n, b, &HarmJob::b_mom);
    const HarmJob& h = J[js >> 1];
    const int k = js & 1;
    hm_moments_tc(h.pts[k], h.units[k], h.n_units[k], h.K, (float)h.delta, h.lmb, h.cr, h.nmm,
                  reinterpret_cast<float2*>(scratch + h.s_MP[k]), b - h.b_mom[k]);
}

__global__ void __launch_bounds__(kFitThreads) hm_groups_jobs(const HarmJob* __restrict__ J, int n,
                                                              char* __restrict__ scratch) {
    const int64_t b = blockIdx.x;
    const int js = set_of(J, n, b, &HarmJob::b_grp);
    const HarmJob& h = J[js >> 1];
    const int k = js & 1;
    const int64_t e = (b - h.b_grp[k]) * kFitThreads + threadIdx.x;
    hm_groups(reinterpret_cast<const float2*>(scratch + h.s_MP[k]), h.gu[k], h.groups[k], h.lmb, h.G[k], h.K,
              reinterpret_cast<float2*>(scratch + h.s_M[k]), e);
}

__global__ void __launch_bounds__(kContractK * kContractWarps) hm_contract_jobs(const HarmJob* __restrict__ J, int n,
                                                                               char* __restrict__ scratch) {
    const int js = set_of(J, n, blockIdx.x, &HarmJob::b_con);
    const HarmJob& h = J[js >> 1];
    const int k = js & 1;
    const int64_t local = (int64_t)blockIdx.x - h.b_con[k];
    const int gx = (h.K + kContractK - 1) / kContractK;
    hm_contract(reinterpret_cast<const float2*>(scratch + h.s_M[k]), h.groups[k], h.G[k],
                h.T, h.nbins, h.LM, h.K, h.Lp, h.lmax, h.lmb, h.aff,
                reinterpret_cast<float2*>(scratch + h.s_C[k]), (int)(local % gx), (int)(local / gx));
}

__global__ void __launch_bounds__(kSynthThreads) hm_synth_jobs(const HarmJob* __restrict__ J, int n,
                                                               char* __restrict__ scratch, char* __restrict__ grid) {
    const HarmJob& h = J[job_of(J, n, blockIdx.x, &HarmJob::b_syn)];
    const int64_t local = (int64_t)blockIdx.x - h.b_syn;
    const int gx = synth_groups(h.Lp);
    hm_synth(h.Lp, reinterpret_cast<const float2*>(scratch + h.s_C[0]),
             h.vox ? reinterpret_cast<const float2*>(scratch + h.s_C[1]) : nullptr, h.K, h.lmax, h.ab, h.nmm, h.step,
             h.vox_s, h.cx, h.cy, h.cz, h.use_center, h.scale, h.origin,
             h.grid_ptr ? h.grid_ptr : reinterpret_cast<float4*>(grid + h.grid_off), (int)(local % gx),
             (int)(local / gx));
}

}  // namespace

int harmonic_max_l() { return kMaxL - 17; }
int harmonic_nodes() { return kNodes; }

namespace {
// Dynamic shared memory of hm_moments: running sums of at most LM + 5 orders
// (a unit's quartet pair) x 24 values.
size_t moments_smem(int LM) { return (size_t)(LM + 5) * 24 * sizeof(float2); }
// Dynamic shared memory of hm_synth for shells up to Lp and outer order li:
// the G_m of kSynthRows rows, the phi phases of the outer shell, and the rows
// in flight (rpp x 6i cells with rpp x i <= 256, or two rows of 6i cells).
size_t synth_smem(int Lp, int li) {
    const int nph = 6 * Lp;
    const int nG = 6 * ((li + 5) / 6) + 6 * ((li + 6) / 6);
    const size_t cells = (size_t)6 * (2 * Lp > kSynthThreads ? 2 * Lp : kSynthThreads);
    return ((size_t)kSynthRows * 2 * nG + (size_t)nph + cells) * sizeof(float2);
}
std::mutex g_smem_mu;
size_t g_smem_set[4][64] = {};  // per device: the limits set for hm_moments (TF32), hm_synth, hm_moments_tc, hm_moments (FP16)
std::atomic<int> g_moments_kind{2};
}  // namespace

void set_moments_kernel(int kind) { g_moments_kind.store(kind >= 0 && kind <= 2 ? kind : 2); }
int moments_kernel() { return g_moments_kind.load(); }

cudaError_t harmonic_take_faults(unsigned* flags) {
    unsigned v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_tc_fault, sizeof v);
    if (e != cudaSuccess) return e;
    if (v) {
        const unsigned zero = 0;
        e = cudaMemcpyToSymbol(g_tc_fault, &zero, sizeof zero);
    }
    if (flags) *flags = v;
    return e;
}

cudaError_t launch_pipe_probe(cudaStream_t s, int kind, int blocks, int iters, float* out) {
    pipe_probe_kernel<<<blocks, 256, 0, s>>>(kind, iters, out);
    return cudaGetLastError();
}

cudaError_t launch_tc_issue_probe(cudaStream_t s, long long* cycles, int* status) {
    constexpr int smem = 1024 + 32768 + 64;
    cudaError_t e = cudaFuncSetAttribute(tc_issue_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    tc_issue_probe_kernel<<<1, 128, smem, s>>>(cycles, status);
    return cudaGetLastError();
}
int tc_issue_probe_mmas() { return kIssueProbeMmas; }

cudaError_t harmonic_reserve_smem(int Lp, int LM) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    const size_t need[4] = {moments_smem(LM), synth_smem(Lp, LM), kTcSmemLaunch, moments_smem(LM)};
    std::lock_guard<std::mutex> lock(g_smem_mu);
    for (int k = 0; k < 4; ++k) {
        if (need[k] <= 48 * 1024 || need[k] <= g_smem_set[k][dev]) continue;
        const void* f = k == 0 ? (const void*)hm_moments_jobs<false>
                        : k == 1 ? (const void*)hm_synth_jobs
                        : k == 2 ? (const void*)hm_moments_tc_jobs
                                 : (const void*)hm_moments_jobs<true>;
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need[k]);
        if (e != cudaSuccess) return e;
        g_smem_set[k][dev] = need[k];
    }
    return cudaSuccess;
}

int harmonic_max_bins() { return kMaxBins; }

cudaError_t launch_radial_tables(cudaStream_t s, const RadialTableArgs& a) {
    const int64_t nodes = (int64_t)a.Lp * a.nbins * kNodes, fits = (int64_t)a.Lp * a.nbins * (a.LM + 1);
    if (nodes <= 0) return cudaSuccess;
    if ((nodes + kNodesThreads - 1) / kNodesThreads > 0x7fffffff || (fits + kFitThreads - 1) / kFitThreads > 0x7fffffff)
        return cudaErrorInvalidValue;
    // rows of shell 0 (never read) stay as they are; shells 1..Lp are written
    hm_nodes_plan<<<(unsigned)((nodes + kNodesThreads - 1) / kNodesThreads), kNodesThreads, 0, s>>>(a);
    hm_fit_plan<<<(unsigned)((fits + kFitThreads - 1) / kFitThreads), kFitThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_voxel_prepare(cudaStream_t s, const VoxelPrepArgs& a) {
    if (a.nb <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.scal, 0, 3 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    vx_prepare<<<(unsigned)((a.nb + kBinThreads - 1) / kBinThreads), kBinThreads, 0, s>>>(
        a.raw, a.nb, a.cx, a.cy, a.cz, a.vs, a.boxes, a.counts, a.scal);
    return cudaGetLastError();
}

cudaError_t launch_voxel_bins(cudaStream_t s, const VoxelBinArgs& a) {
    const int nblk = (int)((a.nv + kBinThreads - 1) / kBinThreads);
    if (a.nbins > kMaxBins) return cudaErrorInvalidValue;
    const int runs = (int)((a.nb + kVstartRun - 1) / kVstartRun);
    vx_run_sums<<<runs, kBinThreads, 0, s>>>(a.counts, a.nb, a.run_sums);
    vx_vstart<<<runs, kBinThreads, 0, s>>>(a.counts, a.nb, a.run_sums, a.vstart);
    vx_expand<<<nblk, kBinThreads, 0, s>>>(a.boxes, a.vstart, a.nb, a.nv, a.vs, a.delta, a.nbins, a.tmp, a.vbin,
                                           a.hist, nblk);
    vx_totals<<<a.nbins, kBinThreads, 0, s>>>(a.hist, a.nbins, nblk, a.total);
    vx_offsets<<<a.nbins, kBinThreads, 0, s>>>(a.hist, a.total, a.nbins, nblk, a.off);
    vx_scatter<<<nblk, kBinThreads, 0, s>>>(a.tmp, a.vbin, a.nv, a.nbins, nblk, a.off, a.out);
    return cudaGetLastError();
}


HarmShape plan_harmonic_jobs(HarmJob* J, int n) {
    HarmShape sh{};
    sh.moments_kind = moments_kernel();
    for (int j = 0; j < n; ++j) {
        HarmJob& h = J[j];
        const int pairs = ((h.LM + 4) / 4 + 1) / 2;
        const int64_t gx = (h.K + kContractK - 1) / kContractK, gy = (h.Lp + kContractShells - 1) / kContractShells;
        for (int k = 0; k < 2; ++k) {
            h.b_mom[k] = sh.moments;
            sh.moments += sh.moments_kind == 0 ? (int64_t)h.n_parts[k] : (int64_t)h.n_units[k] * pairs;
            h.b_grp[k] = sh.groups;
            sh.groups += ((int64_t)h.G[k] * kNodes * h.K + kFitThreads - 1) / kFitThreads;
            h.b_con[k] = sh.contract;
            if (k == 0 || h.vox) sh.contract += gx * gy;  // the coefficient sets the synthesis reads
        }
        h.b_syn = sh.synth;
        sh.synth += (int64_t)((3 * h.Lp / 2 + 1 + kSynthRows - 1) / kSynthRows) * h.Lp;
        sh.maxLp = std::max(sh.maxLp, h.Lp);
        sh.maxLM = std::max(sh.maxLM, h.LM);
    }
    // the launches size their shared memory for the table's largest shell count
    // and order together, which can exceed what any one job's plan reserved
    if (n > 0) sh.reserve_error = harmonic_reserve_smem(sh.maxLp, sh.maxLM);
    return sh;
}

int harmonic_launches_per_batch() { return 4; }

cudaError_t launch_harmonic_jobs(cudaStream_t s, const HarmJob* d_jobs, int n, const HarmShape& sh, char* scratch,
                                 char* grid, cudaEvent_t* ev) {
    if (n <= 0) return cudaSuccess;
    if (sh.reserve_error != cudaSuccess) return sh.reserve_error;
    if (sh.moments > 0x7fffffff || sh.groups > 0x7fffffff || sh.contract > 0x7fffffff || sh.synth > 0x7fffffff)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaSuccess;
    // the limits were raised by harmonic_reserve_smem when the jobs were planned
    if (ev && ev[0]) e = cudaEventRecord(ev[0], s);
    if (e == cudaSuccess && sh.moments > 0) {
        if (sh.moments_kind == 0)
            hm_moments_tc_jobs<<<(unsigned)sh.moments, kTcThreads, kTcSmemLaunch, s>>>(d_jobs, n, scratch);
        else if (sh.moments_kind == 2)
            hm_moments_jobs<true><<<(unsigned)sh.moments, 32, moments_smem(sh.maxLM), s>>>(d_jobs, n, scratch);
        else
            hm_moments_jobs<false><<<(unsigned)sh.moments, 32, moments_smem(sh.maxLM), s>>>(d_jobs, n, scratch);
    }
    if (e == cudaSuccess && ev && ev[1]) e = cudaEventRecord(ev[1], s);
    if (e == cudaSuccess && sh.groups > 0) hm_groups_jobs<<<(unsigned)sh.groups, kFitThreads, 0, s>>>(d_jobs, n, scratch);
    if (e == cudaSuccess && sh.contract > 0)
        hm_contract_jobs<<<(unsigned)sh.contract, kContractK * kContractWarps, 0, s>>>(d_jobs, n, scratch);
    if (e == cudaSuccess && ev && ev[2]) e = cudaEventRecord(ev[2], s);
    if (e == cudaSuccess && sh.synth > 0)
        hm_synth_jobs<<<(unsigned)sh.synth, kSynthThreads, synth_smem(sh.maxLp, sh.maxLM), s>>>(d_jobs, n, scratch,
                                                                                                grid);
    if (e == cudaSuccess && ev && ev[3]) e = cudaEventRecord(ev[3], s);
    return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace dpx
