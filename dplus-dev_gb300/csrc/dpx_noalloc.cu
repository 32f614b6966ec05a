// dpx_noalloc.cu — the orientation average without any device allocation.
//
// Some callers cannot call cudaMalloc/cudaFree: a host application whose
// device memory is entirely pre-reserved by its own pool or caching allocator,
// or a latency-bound serving loop in which a cudaFree (which synchronizes the
// whole device) would stall every other stream.  dpx_mc_average_noalloc gives
// them the Monte Carlo orientation average of one device-resident grid using
// only the memory they pass in plus one fixed scratch array compiled into this
// library: a file-scope __device__ array of DPX_NOALLOC_SCRATCH_BYTES, which
// every GPU that loads libdpx holds until the process exits.
//
// The kernels are the same as dpx_orientation_average's; only where their
// bracket tables and per-chunk partial sums live differs.
#include "dpx.h"
#include "dpx_host.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

namespace {

constexpr size_t kScratchBytes = DPX_NOALLOC_SCRATCH_BYTES;

// Shared by every call on a device; keeps the previous call's contents.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device addresses of g_noalloc_scratch, looked up once per device with that
// device current.  In host code the symbol's name is only a host-side handle,
// never a device address, so kernels receive the looked-up pointer.
constexpr int kMaxDevices = 256;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

int scratch_for_current_device(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return dpx::set_error(DPX_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return dpx::set_error(DPX_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return dpx::set_error(DPX_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e)
                                                                  : "scratch symbol has no device address");
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return DPX_OK;
}

// |A(0)|^2 from the grid origin into res[0] (Amplitude.cpp:1176-1182).
__global__ void origin_kernel(const void* grid, int fp64, double* res) {
    double re, im;
    if (fp64) {
        const double* g = static_cast<const double*>(grid);
        re = g[0];
        im = g[1];
    } else {
        const float* g = static_cast<const float*>(grid);
        re = g[0];
        im = g[1];
    }
    res[0] = re * re + im * im;
}

inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

}  // namespace

extern "C" int dpx_mc_average_noalloc(const void* grid_cells, int grid_size, double qmax, int precision, int nq,
                                      const double* Q, const double* dirs, int64_t n_samples, double eps,
                                      double* res, void* stream) {
    if (!grid_cells || !Q || !dirs || !res) return dpx::set_error(DPX_ERR_ARG, "NULL argument");
    if (grid_size < 2 || (grid_size & 1)) return dpx::set_error(DPX_ERR_ARG, "grid_size must be even and >= 2");
    if (!(qmax > 0)) return dpx::set_error(DPX_ERR_ARG, "qmax must be positive");
    if (precision != DPX_FP32 && precision != DPX_FP64) return dpx::set_error(DPX_ERR_ARG, "bad precision");
    if (nq <= 0 || n_samples <= 0) return dpx::set_error(DPX_ERR_ARG, "nq and n_samples must be positive");
    for (int k = 1; k < nq; ++k)
        if (!(Q[k] >= Q[k - 1])) return dpx::set_error(DPX_ERR_ARG, "Q must be ascending");
    if (!(Q[0] >= 0)) return dpx::set_error(DPX_ERR_ARG, "negative q");
    const dpx::Geom G = dpx::make_geom(grid_size, qmax);
    if (Q[nq - 1] > G.L * G.step * (1.0 + 1e-12)) return dpx::set_error(DPX_ERR_ARG, "q beyond the grid's qmax");

    // bracket tables, as dpx_orientation_average builds them
    dpxh::Brackets B;
    dpxh::make_brackets(G, grid_size, qmax, nq, Q, B);
    const std::vector<int>& br_layer = B.layer;
    const std::vector<int>& br_off = B.off;
    const std::vector<int>& br_qidx = B.qidx;
    const std::vector<double>& br_q = B.q;
    const int max_q = B.max_q;
    dpx::AvgPlan plan{};
    plan.n_brackets = (int)br_layer.size();
    plan.max_q = max_q;
    plan.n_samples = n_samples;
    plan.chunk = eps > 0.0 ? 100 : 128;
    plan.chunk_off = eps > 0.0 ? 99 : 0;
    plan.n_chunks = (n_samples + plan.chunk_off + plan.chunk - 1) / plan.chunk;
    plan.dir_stride = 0;
    plan.dirs = dirs;

    // scratch layout: [q][layer][offsets][q index][model][partial sums + finalize scratch]
    const size_t oQ = 0;
    const size_t oL = align16(oQ + br_q.size() * sizeof(double));
    const size_t oO = align16(oL + br_layer.size() * sizeof(int));
    const size_t oI = align16(oO + br_off.size() * sizeof(int));
    const size_t oM = align16(oI + br_qidx.size() * sizeof(int));
    const size_t oP = (oM + sizeof(dpx::ModelDev) + 255) & ~size_t(255);
    const size_t partial_doubles = ((size_t)plan.n_brackets * (size_t)plan.n_chunks + 5 * (size_t)plan.n_brackets) *
                                   (size_t)max_q;
    const size_t need = oP + partial_doubles * sizeof(double);
    if (need > kScratchBytes) {
        char msg[160];
        snprintf(msg, sizeof msg, "needs %zu bytes of scratch; the static limit is %zu (reduce n_samples or q points)",
                 need, kScratchBytes);
        return dpx::set_error(DPX_ERR_ARG, msg);
    }

    void* scratch = nullptr;
    if (int rc = scratch_for_current_device(&scratch)) return rc;
    char* base = static_cast<char*>(scratch);

    dpx::ModelDev md{};
    md.grid = grid_cells;
    md.R[0] = md.R[4] = md.R[8] = 1.0;
    md.n_groups = 0;
    md.sym_scale = 1.0;
    md.plain = 1;
    plan.need_dir = 0;
    plan.one_leaf = 1;
    std::vector<char> stage(oP);
    std::memcpy(stage.data() + oQ, br_q.data(), br_q.size() * sizeof(double));
    std::memcpy(stage.data() + oL, br_layer.data(), br_layer.size() * sizeof(int));
    std::memcpy(stage.data() + oO, br_off.data(), br_off.size() * sizeof(int));
    std::memcpy(stage.data() + oI, br_qidx.data(), br_qidx.size() * sizeof(int));
    std::memcpy(stage.data() + oM, &md, sizeof md);
    plan.br_q = reinterpret_cast<const double*>(base + oQ);
    plan.br_layer = reinterpret_cast<const int*>(base + oL);
    plan.br_q_off = reinterpret_cast<const int*>(base + oO);
    plan.br_qidx = reinterpret_cast<const int*>(base + oI);
    plan.partial = reinterpret_cast<double*>(base + oP);

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // every result slot starts at zero; the tables are overwritten in full, and the
    // kernels write every partial sum and finalize slot before reading it
    cudaError_t e = cudaMemsetAsync(res, 0, (size_t)nq * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base, stage.data(), oP, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = dpx::launch_average(s, precision == DPX_FP64, G, 1, reinterpret_cast<const dpx::ModelDev*>(base + oM),
                                plan);
    if (e == cudaSuccess) e = dpx::launch_finalize(s, plan, eps, res);
    if (e == cudaSuccess && Q[0] == 0.0) {
        origin_kernel<<<1, 1, 0, s>>>(grid_cells, precision == DPX_FP64, res);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return dpx::set_error(DPX_ERR_CUDA, cudaGetErrorString(e));
    // the staging buffer is pageable: the copy has left it before cudaMemcpyAsync returned
    return DPX_OK;
}
