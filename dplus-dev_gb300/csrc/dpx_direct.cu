// dpx_direct.cu — the FP64 direct-sum orientation average (no grid).
//
// Every grid result is an approximation of the amplitude the reference's
// PDBAmplitude::calcAmplitude (Backend/Backend/PDBAmplitude.cpp:243-317)
// evaluates point by point: the grid's interpolation and, on the FP32 path,
// the bulk precision both err.  dpx_direct_intensity evaluates that amplitude
// with no grid, every step in FP64, at the caller's q values and directions:
//
//   F(q n) = scale [ sum_u aff_u(q) sum_{j in u} e^{i q n.r_j}
//                  + sum_b w_b prod_a L_a sinc(q n_a L_a / 2) e^{i q n.c_b} ]
//
// (the solvent boxes as PDBAmplitude.cpp:277-314), for docked copies
// sum_c e^{i q n.t_c} F(q R_c^T n) (ManualSymmetry, Symmetries.cpp:1079-1166),
// and I(q) = (1/D) sum_d |F(q n_d)|^2 over the given directions.  It is the
// error reference the batch, the server and the bench report against.
//
// Layout: one block per (direction, chunk of up to kQ q values); the block's
// threads stride over (copy, point) and keep kQ complex FP64 sums in
// registers; the block reduces them in a fixed order into partial[d][q]; a
// second kernel sums |partial|^2 over the directions in a fixed order.  The
// result is deterministic.
#include "dpx_host.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr int kQ = 8;         // q values per block
constexpr int kThreads = 256;

struct __align__(32) Pt {
    double x, y, z, w;
};

struct DirectArgs {
    const Pt* pts;   // atoms: x, y, z (nm), ion index
    int64_t n_pts;
    const double* boxes;  // [n_boxes][8]: cx, cy, cz, w, Lx, Ly, Lz, 0
    int64_t n_boxes;
    const double* aff;    // [nq][U] form factors at the q values
    int U;
    const double* Q;
    int nq;
    const double* dirs;   // [D][2] theta, phi
    int64_t D;
    const double* R;      // [9 C] copy rotations (row-major), C = 0: the leaf as given
    const double* T;      // [3 C] copy translations (nm)
    int C;
    double scale;
    double2* partial;     // [D][nq]
};

__device__ inline double sinc(double x) { return x == 0.0 ? 1.0 : sin(x) / x; }

__global__ void __launch_bounds__(kThreads) direct_amp_kernel(DirectArgs a) {
    const int64_t d = blockIdx.x;
    const int q0 = blockIdx.y * kQ;
    const int nqb = min(kQ, a.nq - q0);
    double st, ct, sp, cp;
    sincos(a.dirs[2 * d], &st, &ct);
    sincos(a.dirs[2 * d + 1], &sp, &cp);
    const double n[3] = {st * cp, st * sp, ct};
    double q[kQ];
#pragma unroll
    for (int k = 0; k < kQ; ++k) q[k] = k < nqb ? a.Q[q0 + k] : 0.0;
    double re[kQ], im[kQ];
#pragma unroll
    for (int k = 0; k < kQ; ++k) re[k] = im[k] = 0.0;
    const int copies = a.C > 0 ? a.C : 1;
    for (int c = 0; c < copies; ++c) {
        // n_c = R_c^T n: the direction in the copy's frame; the copy's phase n.t_c
        double nc[3] = {n[0], n[1], n[2]}, tph = 0.0;
        if (a.C > 0) {
            const double* R = a.R + 9 * c;
            for (int i = 0; i < 3; ++i) nc[i] = n[0] * R[i] + n[1] * R[3 + i] + n[2] * R[6 + i];
            tph = n[0] * a.T[3 * c] + n[1] * a.T[3 * c + 1] + n[2] * a.T[3 * c + 2];
        }
        for (int64_t j = threadIdx.x; j < a.n_pts; j += kThreads) {
            const Pt p = a.pts[j];
            const double ph = nc[0] * p.x + nc[1] * p.y + nc[2] * p.z + tph;
            const int u = (int)p.w;
#pragma unroll
            for (int k = 0; k < kQ; ++k) {
                if (k < nqb) {
                    double s, co;
                    sincos(q[k] * ph, &s, &co);
                    const double f = a.aff[(size_t)(q0 + k) * a.U + u];
                    re[k] = fma(f, co, re[k]);
                    im[k] = fma(f, s, im[k]);
                }
            }
        }
        for (int64_t b = threadIdx.x; b < a.n_boxes; b += kThreads) {
            const double* B = a.boxes + 8 * b;
            const double ph = nc[0] * B[0] + nc[1] * B[1] + nc[2] * B[2] + tph;
#pragma unroll
            for (int k = 0; k < kQ; ++k) {
                if (k < nqb) {
                    double v = B[3];
                    for (int ax = 0; ax < 3; ++ax) v *= B[4 + ax] * sinc(0.5 * q[k] * nc[ax] * B[4 + ax]);
                    double s, co;
                    sincos(q[k] * ph, &s, &co);
                    re[k] = fma(v, co, re[k]);
                    im[k] = fma(v, s, im[k]);
                }
            }
        }
    }
    // fixed-order block reduction: warp shuffles, then the warps' sums in order
    __shared__ double2 red[kThreads / 32][kQ];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kQ; ++k) {
        double r = re[k], i = im[k];
        for (int o = 16; o > 0; o >>= 1) {
            r += __shfl_down_sync(0xffffffffu, r, o);
            i += __shfl_down_sync(0xffffffffu, i, o);
        }
        if (lane == 0) red[warp][k] = make_double2(r, i);
    }
    __syncthreads();
    if (threadIdx.x < nqb) {
        double r = 0.0, i = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) {
            r += red[w][threadIdx.x].x;
            i += red[w][threadIdx.x].y;
        }
        a.partial[d * a.nq + q0 + threadIdx.x] = make_double2(a.scale * r, a.scale * i);
    }
}

// I(q) = (1/D) sum_d |partial[d][q]|^2, one block per q, in a fixed order.
__global__ void __launch_bounds__(kThreads) direct_mean_kernel(const double2* partial, int64_t D, int nq,
                                                               double* out) {
    const int k = blockIdx.x;
    double acc = 0.0;
    for (int64_t d = threadIdx.x; d < D; d += kThreads) {
        const double2 f = partial[d * nq + k];
        acc = fma(f.x, f.x, fma(f.y, f.y, acc));
    }
    __shared__ double red[kThreads];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = red[0] / (double)D;
}

}  // namespace

using namespace dpxh;

extern "C" int dpx_direct_intensity(dpx_ctx ctx, const dpx_pdb_desc* d, int n_copies, const double* copy_rot,
                                    const double* copy_tr, int nq, const double* Q, int64_t D, const double* dirs,
                                    double* res) {
    if (!ctx || !d || !Q || !dirs || !res) return fail(DPX_ERR_ARG, "NULL argument");
    if (int rc = check_pdb(*d)) return rc;
    if (d->atoms_on_device) return fail(DPX_ERR_ARG, "the direct sum takes host atoms");
    if (d->aff) return fail(DPX_ERR_ARG, "the direct sum needs the form-factor coefficients, not a table");
    if (nq <= 0 || D <= 0) return fail(DPX_ERR_ARG, "nq and D must be positive");
    if (D > INT32_MAX) return fail(DPX_ERR_ARG, "too many directions");
    if (n_copies < 0 || (n_copies > 0 && (!copy_rot || !copy_tr))) return fail(DPX_ERR_ARG, "bad copy list");
    for (int k = 0; k < nq; ++k)
        if (!(Q[k] >= 0.0)) return fail(DPX_ERR_ARG, "negative q");
    if (int rc = set_device(ctx)) return rc;
    const int U = d->n_ions;
    const int64_t N = d->n_atoms;
    const int64_t nb = d->n_boxes > 0 && d->boxes ? d->n_boxes : 0;
    const int C = n_copies;
    // host staging: points, boxes, form factors, q, directions, copies
    std::vector<double> aff_u;  // [U][nq]
    aff_at(U, d->atoms_per_ion, d->coeffs, d->ion_rads, d->flags, d->solvent_ed, d->c1, nq, Q, aff_u);
    std::vector<double> aff((size_t)nq * U);
    for (int u = 0; u < U; ++u)
        for (int k = 0; k < nq; ++k) aff[(size_t)k * U + u] = aff_u[(size_t)u * nq + k];
    std::vector<Pt> pts(N);
    {
        int64_t j = 0;
        for (int u = 0; u < U; ++u)
            for (int i = 0; i < d->atoms_per_ion[u]; ++i, ++j)
                pts[j] = Pt{d->atoms[4 * j], d->atoms[4 * j + 1], d->atoms[4 * j + 2], (double)u};
    }
    std::vector<double> boxes((size_t)8 * nb);
    for (int64_t i = 0; i < 8 * nb; ++i) boxes[i] = d->boxes[i];
    std::vector<double> R((size_t)9 * C), T((size_t)3 * C);
    for (int c = 0; c < C; ++c) {
        euler(copy_rot[3 * c], copy_rot[3 * c + 1], copy_rot[3 * c + 2], &R[9 * c]);
        for (int k = 0; k < 3; ++k) T[3 * c + k] = copy_tr[3 * c + k];
    }
    std::vector<char> h;
    auto put = [&](const void* src, size_t n) {
        const size_t at = al16(h.size());
        h.resize(at + n);
        if (n) std::memcpy(h.data() + at, src, n);
        return at;
    };
    const size_t oP = put(pts.data(), pts.size() * sizeof(Pt));
    const size_t oB = put(boxes.data(), boxes.size() * sizeof(double));
    const size_t oA = put(aff.data(), aff.size() * sizeof(double));
    const size_t oQ = put(Q, (size_t)nq * sizeof(double));
    const size_t oD = put(dirs, (size_t)D * 2 * sizeof(double));
    const size_t oR = put(R.data(), R.size() * sizeof(double));
    const size_t oT = put(T.data(), T.size() * sizeof(double));
    const size_t oPart = al16(h.size());
    const size_t oOut = al16(oPart + (size_t)D * nq * sizeof(double2));
    const size_t total = oOut + (size_t)nq * sizeof(double);
    if (cudaError_t e = ctx->direct.reserve(total)) {
        cudaGetLastError();
        return fail(DPX_ERR_OOM, "direct sum needs %zu bytes (%s)", total, cudaGetErrorString(e));
    }
    char* base = static_cast<char*>(ctx->direct.p);
    cudaStream_t s = ctx->stream;
    DPX_CUDA(cudaMemcpyAsync(base, h.data(), h.size(), cudaMemcpyHostToDevice, s));
    DirectArgs a{};
    a.pts = reinterpret_cast<const Pt*>(base + oP);
    a.n_pts = N;
    a.boxes = reinterpret_cast<const double*>(base + oB);
    a.n_boxes = nb;
    a.aff = reinterpret_cast<const double*>(base + oA);
    a.U = U;
    a.Q = reinterpret_cast<const double*>(base + oQ);
    a.nq = nq;
    a.dirs = reinterpret_cast<const double*>(base + oD);
    a.D = D;
    a.R = reinterpret_cast<const double*>(base + oR);
    a.T = reinterpret_cast<const double*>(base + oT);
    a.C = C;
    a.scale = d->scale;
    a.partial = reinterpret_cast<double2*>(base + oPart);
    double* out = reinterpret_cast<double*>(base + oOut);
    direct_amp_kernel<<<dim3((unsigned)D, (unsigned)((nq + kQ - 1) / kQ)), kThreads, 0, s>>>(a);
    DPX_CUDA(cudaGetLastError());
    direct_mean_kernel<<<nq, kThreads, 0, s>>>(a.partial, D, nq, out);
    DPX_CUDA(cudaGetLastError());
    DPX_CUDA(cudaMemcpyAsync(res, out, (size_t)nq * sizeof(double), cudaMemcpyDeviceToHost, s));
    DPX_CUDA(cudaStreamSynchronize(s));
    return DPX_OK;
}
