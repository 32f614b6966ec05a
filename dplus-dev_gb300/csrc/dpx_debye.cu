// dpx_debye.cu — the Debye sum of a PDB leaf, an orientation average that
// needs no grid:
//   I(q) = sum_i |f_i|^2 + 2 sum_{i<j} Re(f_i conj f_j) sin(q r_ij) / (q r_ij)
// (DebyeCalTester::Calculate, PDBAmplitude.cpp:1789-1825; GPU kernels
// Debye32x32 / DebyeMapsV4, DebyeCalculator.cu:60-160, 415-484).
//
// GB300 layout: the reference launches one kernel per q value and rebuilds the
// per-atom form factors on the host for every q.  Here one launch covers every
// q: a block takes MQ = 16 q values and a pair of 128-atom tile rows (row a and
// row T-1-a, so every block sees T+1 tiles of the lower triangle), stages the
// j tile (positions and the per-atom form factors of its 16 q values) in
// shared memory and each thread sums its own atom i against it.  Per (pair, q)
// the FP32 path costs one SFU sine and about a dozen FMA-pipe operations: the
// FMA pipe bounds it.  Per-atom form factors F[q][atom] (ion form factor minus
// the dummy-atom solvent, plus f' + i f'', times the Debye-Waller factor) are
// built once by a table kernel; the diagonal terms and the per-block partial
// sums are reduced in FP64 in a fixed order, so results are reproducible.
#include "dpx_internal.h"

namespace dpx {
namespace {

constexpr int kTile = 128;  // atoms per tile = threads per block
constexpr int kMQ = 16;     // q values per block

// sin(x) / x for x >= 0 given 1/x, FP32.  Below x = 0.5 the Taylor series
// (truncation < 1.1e-8); above, x is reduced to [-pi, pi] (n = round(x / 2pi)
// by the 1.5 * 2^23 shift, 2pi in two parts as Cody and Waite do) and the SFU
// sine, whose absolute error there is about 4e-7, is divided by x.
__device__ __forceinline__ float debye_sinc(float x, float inv_x) {
    const float x2 = x * x;
    const float n = fmaf(x, 0.159154943091895336f, 12582912.f) - 12582912.f;
    float y = fmaf(-n, 6.28125f, x);
    y = fmaf(-n, 1.93530717958647692e-3f, y);
    const float big = __sinf(y) * inv_x;
    const float small = fmaf(x2, fmaf(x2, fmaf(x2, -1.f / 5040.f, 1.f / 120.f), -1.f / 6.f), 1.f);
    return x2 < 0.25f ? small : big;
}

__device__ __forceinline__ double debye_sinc(double x, double) { return x == 0.0 ? 1.0 : sin(x) / x; }

template <typename T>
__device__ __forceinline__ T pair_distance(float4 a, float4 b, T& inv_r);

template <>
__device__ __forceinline__ float pair_distance<float>(float4 a, float4 b, float& inv_r) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float ir = rsqrtf(d2);
    inv_r = d2 > 0.f ? ir : 0.f;
    return d2 * inv_r;
}

template <>
__device__ __forceinline__ double pair_distance<double>(float4 a, float4 b, double& inv_r) {
    const double dx = (double)a.x - (double)b.x, dy = (double)a.y - (double)b.y, dz = (double)a.z - (double)b.z;
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    inv_r = r > 0.0 ? 1.0 / r : 0.0;
    return r;
}

// F[k][i] = (ff[ion_i][k] + f'_i + i f''_i) exp(-B_i (q_k / 10)^2 / (16 pi^2)),
// zero for the padding atoms i >= n.
template <typename T, bool ANOM>
__global__ void debye_ff_kernel(const double* __restrict__ ff, const int* __restrict__ ion, const float* __restrict__ bf,
                                const float2* __restrict__ anom, const double* __restrict__ q, int nq, int64_t n,
                                int64_t npad, T* __restrict__ Fr, T* __restrict__ Fi) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    for (int k = blockIdx.y; k < nq; k += gridDim.y) {
        double re = 0.0, im = 0.0;
        if (i < n) {
            re = ff[(int64_t)ion[i] * nq + k];
            if (ANOM) {
                re += (double)anom[i].x;
                im = (double)anom[i].y;
            }
            if (bf) {
                const double q10 = q[k] / 10.0;
                const double dw = exp(-((double)bf[i] * q10 * q10 / (16.0 * 9.86960440108935861883)));
                re *= dw;
                im *= dw;
            }
        }
        Fr[(int64_t)k * npad + i] = (T)re;
        if (ANOM) Fi[(int64_t)k * npad + i] = (T)im;
    }
}

template <typename T, bool ANOM>
__global__ void __launch_bounds__(kTile) debye_pairs_kernel(const float4* __restrict__ pos, const T* __restrict__ Fr,
                                                            const T* __restrict__ Fi, const double* __restrict__ qv,
                                                            int nq, int64_t npad, int n_tiles,
                                                            double* __restrict__ partial) {
    __shared__ float4 s_pos[kTile];
    __shared__ __align__(16) T s_fr[kTile][kMQ];
    __shared__ __align__(16) T s_fi[ANOM ? kTile : 1][kMQ];
    __shared__ double s_red[kTile / 32][kMQ];
    const int t = threadIdx.x;
    const int k0 = blockIdx.y * kMQ;
    const int mq = min(kMQ, nq - k0);
    T q[kMQ], iq[kMQ];
#pragma unroll
    for (int k = 0; k < kMQ; ++k) {
        const double qq = k < mq ? qv[k0 + k] : 0.0;
        q[k] = (T)qq;
        iq[k] = qq > 0.0 ? (T)(1.0 / qq) : T(0);
    }
    double tot[kMQ];
#pragma unroll
    for (int k = 0; k < kMQ; ++k) tot[k] = 0.0;

    for (int pass = 0; pass < 2; ++pass) {
        const int ti = pass == 0 ? (int)blockIdx.x : n_tiles - 1 - (int)blockIdx.x;
        if (pass == 1 && ti <= (int)blockIdx.x) break;
        const int64_t i = (int64_t)ti * kTile + t;
        const float4 pi = pos[i];
        T fri[kMQ], fii[kMQ];
#pragma unroll
        for (int k = 0; k < kMQ; ++k) {
            fri[k] = k < mq ? Fr[(int64_t)(k0 + k) * npad + i] : T(0);
            fii[k] = (ANOM && k < mq) ? Fi[(int64_t)(k0 + k) * npad + i] : T(0);
        }
        for (int tj = 0; tj <= ti; ++tj) {
            const int64_t j0 = (int64_t)tj * kTile;
            __syncthreads();
            s_pos[t] = pos[j0 + t];
#pragma unroll
            for (int k = 0; k < kMQ; ++k) {
                s_fr[t][k] = k < mq ? Fr[(int64_t)(k0 + k) * npad + j0 + t] : T(0);
                if (ANOM) s_fi[t][k] = k < mq ? Fi[(int64_t)(k0 + k) * npad + j0 + t] : T(0);
            }
            __syncthreads();
            T acc[kMQ];
#pragma unroll
            for (int k = 0; k < kMQ; ++k) acc[k] = T(0);
            const int jend = tj == ti ? t : kTile;  // the diagonal tile holds the pairs j < i
            for (int j = 0; j < jend; ++j) {
                T inv_r;
                const T r = pair_distance<T>(pi, s_pos[j], inv_r);
#pragma unroll
                for (int k = 0; k < kMQ; ++k) {
                    const T s = debye_sinc(q[k] * r, inv_r * iq[k]);
                    T w = s_fr[j][k];
                    if (ANOM) w = w * fri[k] + s_fi[j][k] * fii[k];
                    acc[k] += w * s;
                }
            }
#pragma unroll
            for (int k = 0; k < kMQ; ++k)
                tot[k] += ANOM ? 2.0 * (double)acc[k] : 2.0 * (double)fri[k] * (double)acc[k];
        }
    }
    // block reduction in FP64, fixed order
    const int warp = t >> 5, lane = t & 31;
#pragma unroll
    for (int k = 0; k < kMQ; ++k) {
        double v = tot[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) s_red[warp][k] = v;
    }
    __syncthreads();
    if (t < mq) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kTile / 32; ++w) s += s_red[w][t];
        partial[(int64_t)blockIdx.x * nq + k0 + t] = s;
    }
}

// out[k] = scale^2 (sum_i |F_i|^2 + sum_b partial[b][k]); one block per q.
template <typename T, bool ANOM>
__global__ void debye_finalize_kernel(const T* __restrict__ Fr, const T* __restrict__ Fi, const double* __restrict__ partial,
                                      int n_blocks, int nq, int64_t npad, double scale2, double* __restrict__ out) {
    __shared__ double s_red[8];
    const int k = blockIdx.x;
    double v = 0.0;
    for (int64_t i = threadIdx.x; i < npad; i += blockDim.x) {
        const double a = (double)Fr[(int64_t)k * npad + i];
        v += a * a;
        if (ANOM) {
            const double b = (double)Fi[(int64_t)k * npad + i];
            v += b * b;
        }
    }
    for (int b = threadIdx.x; b < n_blocks; b += blockDim.x) v += partial[(int64_t)b * nq + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += s_red[w];
        out[k] = scale2 * s;
    }
}

template <typename T, bool ANOM>
cudaError_t debye_launch(cudaStream_t s, const DebyeArgs& a) {
    const int n_tiles = (int)(a.npad / kTile);
    const int pair_rows = (n_tiles + 1) / 2;
    T* Fr = reinterpret_cast<T*>(a.Fr);
    T* Fi = reinterpret_cast<T*>(a.Fi);
    debye_ff_kernel<T, ANOM><<<dim3((unsigned)((a.npad + 255) / 256), (unsigned)min(a.nq, 65535)), 256, 0, s>>>(
        a.ff, a.ion, a.bfactor, a.anom, a.q, a.nq, a.n, a.npad, Fr, Fi);
    debye_pairs_kernel<T, ANOM><<<dim3((unsigned)pair_rows, (unsigned)((a.nq + kMQ - 1) / kMQ)), kTile, 0, s>>>(
        a.pos, Fr, Fi, a.q, a.nq, a.npad, n_tiles, a.partial);
    debye_finalize_kernel<T, ANOM><<<a.nq, 256, 0, s>>>(Fr, Fi, a.partial, pair_rows, a.nq, a.npad, a.scale2, a.out);
    return cudaGetLastError();
}

}  // namespace

int64_t debye_padded_atoms(int64_t n) { return (n + kTile - 1) / kTile * kTile; }
int debye_pair_blocks(int64_t npad) { return (int)((npad / kTile + 1) / 2); }

cudaError_t launch_debye(cudaStream_t s, bool fp64, bool anomalous, const DebyeArgs& a) {
    if (a.nq <= 0 || a.n <= 0) return cudaSuccess;
    if (fp64) return anomalous ? debye_launch<double, true>(s, a) : debye_launch<double, false>(s, a);
    return anomalous ? debye_launch<float, true>(s, a) : debye_launch<float, false>(s, a);
}

}  // namespace dpx
