// kg_device.cuh -- device pointer bundle and small device helpers shared by the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "kg_internal.h"

namespace kg {

constexpr int BLOCK = 256;           // threads per CTA of every kernel
constexpr int MAX_INC = 24;          // incidences a cell may hold (checked on the host)
constexpr double JL_EPS = 2.220446049250313e-16;   // Julia eps()
constexpr double EPS_REF = 1e-12;                  // EPS (src/Abstract/Types.jl:3)
constexpr double PI = 3.141592653589793;

// status word bits written by the kernels (mapped to KG_ERR_* on the host)
constexpr int ST_NONFINITE = 1;
constexpr int ST_NEGATIVE = 2;
constexpr int RES_STRIDE = 2 * MAXW + 2;   // per slot: sums, checked step, checked flag
constexpr int MAX_SLOTS = 4096;            // problems a handle can hold

struct Dev {
    int dim, ndf, n_cells, n_walls;
    int64_t PG;                        // total velocity cells over all grids
    // grids
    const int64_t* g_off;
    const int8_t* vlev;
    const double* vw;
    const double* vu;                  // [dim][PG]
    const float* vuf;                  // FP32 copies (mixed form)
    const float* vwf;
    const int32_t* ax_off;             // axis tables of the factorised Maxwellian
    const double* ax_val;
    const uint16_t* vidx;
    int max_axis;
    // data table
    const int64_t* foff;
    const int32_t* dgrid;
    const int32_t* dbe;
    const double* dmid;                // [n_data][MAXD]
    const double* dds;
    // pairings
    const int64_t* p_off;
    const int32_t* p_j0;
    const int32_t* p_cnt;
    // slope
    const SlopeOp* slope_ops;
    const int32_t* pass_cells;
    const int32_t* cell_slope_op;
    const NbrRef* slope_nbr;
    // flux
    const int32_t* fluid_cells;
    const int32_t* inc_off;
    const Incidence* inc;
    const double* bc_prim;
    // ib
    const SolidOp* solid_ops;
    const WallOp* wall_ops;
    const NbrRef* ib_nbr;
    const double* ib_dx;
    const int32_t* cut_idx;
    const double* cut_gw;
    const double* cut_sw;
    const double* cvcw;
    // problems: per data item its slot; per slot the parameters and the step counter
    const int32_t* dnv;
    const int32_t* dprob;
    const ProbParams* probs;
    int64_t* prob_step;
    int flux, marching;
    // state
    void* f_in;                        // T*
    void* f_out;                       // T*
    void* sdf;                         // T*
    double* w;                         // [n_cells][MAXW]
    double* prim;
    double* qf;                        // [n_cells][MAXD]
    double* cell_res;                  // [n_fluid][2*MAXW] residual scratch
    int* status;                       // per slot
};

// ---- reductions --------------------------------------------------------------
// Block sums with a fixed combination order (deterministic run to run): a butterfly
// within each warp, then warp 0 combines the warp partials and broadcasts the result
// through shared memory, so every thread sees the same bits.
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double* sred) {
    // sred: shared scratch of N * (BLOCK/32) doubles
    constexpr int NWARP = BLOCK / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int e = 0; e < N; ++e) {
        double x = v[e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        v[e] = x;
    }
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int e = 0; e < N; ++e) sred[e * NWARP + wid] = v[e];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int e = 0; e < N; ++e) {
            double x = lane < NWARP ? sred[e * NWARP + lane] : 0.0;
#pragma unroll
            for (int o = NWARP / 2; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) sred[e * NWARP] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < N; ++e) v[e] = sred[e * NWARP];
    __syncthreads();
}

// Block sum of FP32 compensated partials (value = hi + lo per thread): the warp butterfly
// combines float-float pairs with TwoSum in FP32; only the warp partials meet FP64.
template <int N>
__device__ __forceinline__ void block_sum_ff(float (&hi)[N], float (&lo)[N], double (&out)[N], double* sred) {
    constexpr int NWARP = BLOCK / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int e = 0; e < N; ++e) {
        float h = hi[e], l = lo[e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float h2 = __shfl_xor_sync(0xffffffffu, h, o);
            const float l2 = __shfl_xor_sync(0xffffffffu, l, o);
            const float sum = h + h2;
            const float bp = sum - h;
            const float err = (h - (sum - bp)) + (h2 - bp);
            l = l + l2 + err;
            h = sum;
        }
        hi[e] = h;
        lo[e] = l;
    }
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int e = 0; e < N; ++e) sred[e * NWARP + wid] = (double)hi[e] + (double)lo[e];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int e = 0; e < N; ++e) {
            double x = lane < NWARP ? sred[e * NWARP + lane] : 0.0;
#pragma unroll
            for (int o = NWARP / 2; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) sred[e * NWARP] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < N; ++e) out[e] = sred[e * NWARP];
    __syncthreads();
}

__device__ __forceinline__ double sgn(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }
__device__ __forceinline__ double minmod(double a, double b) {
    return 0.5 * (sgn(a) + sgn(b)) * fmin(fabs(a), fabs(b));
}
__device__ __forceinline__ float sgnf(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
__device__ __forceinline__ float minmod(float a, float b) {
    return 0.5f * (sgnf(a) + sgnf(b)) * fminf(fabsf(a), fabsf(b));
}

// get_prim_2D / 3D (lib/KitCore/2D.jl:9-16, 3D.jl:12-20)
template <int D>
__device__ __forceinline__ void get_prim(const double* w, double gamma, double* prim) {
    prim[0] = w[0];
    double m2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) { prim[1 + d] = w[1 + d] / w[0]; m2 += w[1 + d] * w[1 + d]; }
    prim[D + 1] = 0.5 * w[0] / (gamma - 1.0) / (w[D + 1] - 0.5 * m2 / w[0]);
}

// scale factor 2^(D*(lj-li)) of the merge walk when the source is finer, else 1
template <int D>
__device__ __forceinline__ double merge_inv_scale(int li, int lj) {
    return lj > li ? ldexp(1.0, -D * (lj - li)) : 1.0;
}

}  // namespace kg
