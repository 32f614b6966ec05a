// dpx_spline.cuh — phi-spline derivative of one cell of a theta row, shared by
// the spline pass (dpx_kernels.cu) and the harmonic synthesis
// (dpx_harmonic.cu) so that both give the same bits.
//
// Periodic cubic-spline derivatives along a row of n cells (D+
// PeriodicSplineSolver.h:7-67, Grid.cpp:1113-1151).  The inverse of the
// circulant circ(1,4,1) is a two-sided geometric kernel G(m) = C(a^m + a^(n-m))
// / (1 - a^n), a = sqrt(3) - 2, C = 1/(2 sqrt 3); folding the right-hand side
// 3(y[k+1]-y[k-1]) into it gives d_k = sum_s H(s) (y[k-s] - y[k+s]) with
// H(s) = 3C a^(s-1) (a^2 - 1).  Long rows use the K-term truncation (|a|^K
// below the type's epsilon); short rows use the exact periodic kernel.
#pragma once

#include <cuda_runtime.h>

namespace dpx {

// d(y)[p] of a periodic row of n cells; get(k) returns cell k's value as a
// type with members x (real) and y (imaginary).
template <typename T, int K, typename Get>
__device__ __forceinline__ void row_spline(int n, int p, Get get, T& dr, T& di) {
    const double alpha = -0.26794919243112270647;  // sqrt(3) - 2
    const double C = 0.28867513459481288225;        // 1 / (2 sqrt 3)
    dr = 0;
    di = 0;
    if (n > 2 * K + 2) {
        double w = 3.0 * C * (alpha * alpha - 1.0);
#pragma unroll
        for (int s = 1; s <= K; ++s) {
            int lo = p - s;
            if (lo < 0) lo += n;
            int hi = p + s;
            if (hi >= n) hi -= n;
            const auto a = get(lo);
            const auto b = get(hi);
            dr += T(w) * (a.x - b.x);
            di += T(w) * (a.y - b.y);
            w *= alpha;
        }
    } else {
        const double an = pow(alpha, (double)n);
        const double denom = 1.0 / (1.0 - an);
        for (int s = 0; s < n; ++s) {
            int m1 = s + 1;
            if (m1 >= n) m1 -= n;
            int m0 = s - 1;
            if (m0 < 0) m0 += n;
            const double g1 = C * (pow(alpha, (double)m1) + pow(alpha, (double)(n - m1))) * denom;
            const double g0 = C * (pow(alpha, (double)m0) + pow(alpha, (double)(n - m0))) * denom;
            const double h = 3.0 * (g1 - g0);
            int k = p - s;
            if (k < 0) k += n;
            const auto a = get(k);
            dr += T(h) * a.x;
            di += T(h) * a.y;
        }
    }
}

}  // namespace dpx
