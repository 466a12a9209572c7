// kg_noalloc.cu -- residual sums without any device allocation.
//
// kg_residual_sums_noalloc computes the two sums of residual_check!
// (Σ_c (prim_new - prim_old)^2 and Σ_c |prim_new|, src/Solver/Finalize.jl:5-11) over
// arrays the caller already holds on the device.  The handle path computes the same sums
// with per-cell terms in a cudaMalloc'd buffer; some callers cannot allocate device
// memory at the point where they need the residual: a host runtime whose device memory
// is owned by its own pool allocator (the Julia caller's CUDA.jl pool), or a serving loop
// that must not let an allocation synchronise the device while other problems' steps are
// in flight.  This entry point keeps its scratch in a fixed file-scope device array
// instead, so it allocates nothing.
//
// Scratch: kg_noalloc_partials holds one row of 2*MAXW partial sums per block, at most
// KG_NOALLOC_MAX_BLOCKS rows (80 KiB); every GPU that loads the library holds it until the
// process exits.  A call covers at most KG_NOALLOC_MAX_CELLS cells and rejects more.
// Calls share the array: two calls that overlap on the GPU (on different streams, or
// from different threads) race on it.  The first pass writes every row the second pass
// reads, so nothing has to start at zero and the contents left by the previous call are
// never read.
#include <cuda_runtime.h>
#include <mutex>
#include <string>
#include "kg_device.cuh"

namespace {

constexpr int KG_NOALLOC_MAX_BLOCKS = 1024;
constexpr int KG_NOALLOC_CELLS_PER_BLOCK = 4096;
constexpr int64_t KG_NOALLOC_MAX_CELLS = (int64_t)KG_NOALLOC_MAX_BLOCKS * KG_NOALLOC_CELLS_PER_BLOCK;
constexpr int ROW = 2 * kg::MAXW;

static __device__ __align__(256) double kg_noalloc_partials[KG_NOALLOC_MAX_BLOCKS * ROW];

// Device address of kg_noalloc_partials per device, resolved once with that device current.
// The cached address belongs to the device's primary context, which this entry point
// assumes lives as long as the process: after a cudaDeviceReset the cached address would
// point into a destroyed context, so a caller must not reset a device it uses this on.
constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
double* g_addr[MAX_DEVICES] = {};

__global__ void __launch_bounds__(kg::BLOCK) partial_kernel(const double* __restrict__ pn, const double* __restrict__ po,
                                                            int64_t n, int nw, double* __restrict__ partials) {
    __shared__ double sred[ROW * (kg::BLOCK / 32)];
    double v[ROW];
#pragma unroll
    for (int q = 0; q < ROW; ++q) v[q] = 0.0;
    const int64_t c0 = (int64_t)blockIdx.x * KG_NOALLOC_CELLS_PER_BLOCK;
    const int64_t c1 = c0 + KG_NOALLOC_CELLS_PER_BLOCK < n ? c0 + KG_NOALLOC_CELLS_PER_BLOCK : n;
    for (int64_t c = c0 + threadIdx.x; c < c1; c += kg::BLOCK) {
        // unrolled over MAXW with a guard, so that v stays in registers
#pragma unroll
        for (int q = 0; q < kg::MAXW; ++q) {
            if (q < nw) {
                const double a = pn[c * nw + q], d = a - po[c * nw + q];
                v[q] += d * d;
                v[kg::MAXW + q] += fabs(a);
            }
        }
    }
    kg::block_sum<ROW>(v, sred);
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < ROW; ++q) partials[(int64_t)blockIdx.x * ROW + q] = v[q];
}

__global__ void __launch_bounds__(kg::BLOCK) final_kernel(const double* __restrict__ partials, int nblocks, int nw,
                                                          double* __restrict__ out) {
    __shared__ double sred[ROW * (kg::BLOCK / 32)];
    double v[ROW];
#pragma unroll
    for (int q = 0; q < ROW; ++q) v[q] = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kg::BLOCK)
#pragma unroll
        for (int q = 0; q < ROW; ++q) v[q] += partials[(int64_t)b * ROW + q];
    kg::block_sum<ROW>(v, sred);
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < kg::MAXW; ++q)
            if (q < nw) { out[q] = v[q]; out[nw + q] = v[kg::MAXW + q]; }
}

}  // namespace

namespace kg {
void set_global_error(const std::string& msg);   // read back by kg_last_error(NULL, ...)
}

extern "C" int kg_residual_sums_noalloc(const double* prim_new, const double* prim_old, int64_t n_cells,
                                        int32_t dim, double* sums, void* stream) {
    if (!prim_new || !prim_old || !sums || (dim != 2 && dim != 3) || n_cells < 0) {
        kg::set_global_error("kg_residual_sums_noalloc: null pointer or bad dim/n_cells");
        return KG_ERR_ARG;
    }
    if (n_cells > KG_NOALLOC_MAX_CELLS) {
        kg::set_global_error("kg_residual_sums_noalloc: n_cells " + std::to_string(n_cells) +
                             " exceeds the maximum " + std::to_string(KG_NOALLOC_MAX_CELLS));
        return KG_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        kg::set_global_error(std::string("kg_residual_sums_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return KG_ERR_CUDA;
    }
    if (dev < 0 || dev >= MAX_DEVICES) {
        kg::set_global_error("kg_residual_sums_noalloc: device index " + std::to_string(dev) +
                             " is outside the " + std::to_string(MAX_DEVICES) + " devices this entry point serves");
        return KG_ERR_ARG;
    }
    double* part = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            // first call on this device: resolve the array's device address (current device)
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, kg_noalloc_partials);
            if (e != cudaSuccess || !p) {
                kg::set_global_error(std::string("kg_residual_sums_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
                return KG_ERR_CUDA;
            }
            g_addr[dev] = (double*)p;
        }
        part = g_addr[dev];
    }
    const int nw = dim + 2;
    int nblocks = (int)((n_cells + KG_NOALLOC_CELLS_PER_BLOCK - 1) / KG_NOALLOC_CELLS_PER_BLOCK);
    cudaStream_t s = (cudaStream_t)stream;
    if (nblocks > 0) partial_kernel<<<nblocks, kg::BLOCK, 0, s>>>(prim_new, prim_old, n_cells, nw, part);
    final_kernel<<<1, kg::BLOCK, 0, s>>>(part, nblocks, nw, sums);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        kg::set_global_error(std::string("kg_residual_sums_noalloc: launch: ") + cudaGetErrorString(e));
        return KG_ERR_CUDA;
    }
    return KG_OK;
}
