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
    const float* ax_hi;                // ax_val as FP32 hi + lo
    const float* ax_lo;
    const uint16_t* vidx;
    int max_axis;
    // data table
    const int64_t* foff;
    const int32_t* dgrid;
    const int32_t* dbe;
    const double* dmid;                // [n_data][MAXD]
    const double* dds;
    const double* dinvv;               // 1 / cell volume
    // pairings
    const int64_t* p_off;
    const int32_t* p_j0;
    const int32_t* p_cnt;
    // slope
    const SlopeOp* slope_ops;
    const int32_t* pass_cells;
    const int32_t* slope_items;        // (pass-cell entry, velocity chunk) per slope CTA
    int slope_split;                   // 0: one item per pass cell, item == pass-cell entry
    int slope_chunk;                   // velocity cells per work item (SLOPE_CHUNK or a whole cell)
    const int32_t* cell_slope_op;
    const NbrRef* slope_nbr;
    // flux
    const int32_t* fluid_cells;
    const uint8_t* fluid_reg;          // per fluid cell: regular (fast path of the flux kernel)
    const FluxCell* fcrec;             // per fluid cell: its record
    const RegRec* regrec;              // per fluid cell: the faces of a regular cell
    const R2Rec* r2rec;                // per fluid cell: R2 cells' neighbours of neighbours
    const SlopeCell* screc;            // per pass-cell entry: its record
    const CritOp* crit_ops;            // per fluid cell and direction (physical-space criterion)
    const int32_t* crit_nbr;
    const int32_t* inc_off;
    const Incidence* inc;
    const double* bc_prim;
    const float* bc_hl;                // bc_prim as FP32 hi (MAXW) then lo (MAXW) per entry
    int max_bcm;                       // most Maxwellian-state domain faces of a cell
    int fst_global;                    // flux kernel: convected f staged in the cell's output
                                       // block (L2) instead of shared memory
    int flux_nt;                       // flux kernel threads per CTA: 256, or 128 for layouts of
                                       // small velocity grids (twice the cells in flight)
    int slope_nt;                      // slope kernel threads per CTA (the same choice)
    int packed_nt;                     // packed kernels' threads per CTA: 64 for layouts of small
                                       // velocity grids (more cells in flight), else flux_nt
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
template <int N, int NT = BLOCK>
__device__ __forceinline__ void block_sum(double (&v)[N], double* sred) {
    // sred: shared scratch of N * (NT/32) doubles; NT: threads of the block
    constexpr int NWARP = NT / 32;
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

// Block sum of FP32 compensated partials (value = hi + lo per thread), all in float-float
// arithmetic: a TwoSum butterfly within each warp, then warp 0 combines the warp partials the
// same way, one lane per warp and element, and one lane per element converts the total to FP64
// (three FP64 instructions per round of elements instead of three per element and warp).
// Fixed combination order: deterministic run to run, and every thread sees the same bits.
__device__ __forceinline__ void two_sum_acc(float& h, float& l, float h2, float l2) {
    const float sum = h + h2;
    const float bp = sum - h;
    const float err = (h - (sum - bp)) + (h2 - bp);
    l = l + l2 + err;
    h = sum;
}
// The warp stage transposes as it sums: with the N elements padded to P = 2^K, each exchange
// at offset 16, 8, ... hands the partner the half of the elements it keeps and adds the half it
// receives, so after K exchanges every lane holds one element (e = lane >> (5 - K)) summed over
// 2^K lanes, and plain butterflies at the remaining offsets finish it: 2 (P - 1) + 2 (5 - K)
// shuffles and P - 1 + 5 - K float-float additions instead of 10 N and 5 N.
template <int N> struct Pow2 { static constexpr int K = N <= 1 ? 0 : N <= 2 ? 1 : N <= 4 ? 2 : N <= 8 ? 3 : N <= 16 ? 4 : 5; };
template <int N, int NT = BLOCK>
__device__ __forceinline__ void block_sum_ff(float (&hi)[N], float (&lo)[N], double (&out)[N], double* sred) {
    // sred: shared scratch of at least N * (NT/32) doubles; NT: threads of the block
    constexpr int NWARP = NT / 32;
    static_assert(NWARP == 2 || NWARP == 4 || NWARP == 8, "the warp-0 stage maps NWARP lanes per element");
    static_assert(N <= 32, "at most 32 elements");
    constexpr int GROUPS = 32 / NWARP;            // elements per round of warp 0
    constexpr int K = Pow2<N>::K, P = 1 << K;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float h[P], l[P];
#pragma unroll
    for (int e = 0; e < P; ++e) { h[e] = e < N ? hi[e] : 0.f; l[e] = e < N ? lo[e] : 0.f; }
#pragma unroll
    for (int s = 0; s < K; ++s) {
        const int o = 16 >> s, c = P >> s, half = c >> 1;
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < half; ++j) {
            const float mh = up ? h[j + half] : h[j], ml = up ? l[j + half] : l[j];
            const float sh = up ? h[j] : h[j + half], sl = up ? l[j] : l[j + half];
            float rh = mh, rl = ml;
            two_sum_acc(rh, rl, __shfl_xor_sync(0xffffffffu, sh, o), __shfl_xor_sync(0xffffffffu, sl, o));
            h[j] = rh;
            l[j] = rl;
        }
    }
#pragma unroll
    for (int o = 16 >> K; o > 0; o >>= 1)
        two_sum_acc(h[0], l[0], __shfl_xor_sync(0xffffffffu, h[0], o), __shfl_xor_sync(0xffffffffu, l[0], o));
    float2* sf = reinterpret_cast<float2*>(sred);   // [N][NWARP] partials
    __syncthreads();
    {
        const int e = lane >> (5 - K);
        if ((lane & ((1 << (5 - K)) - 1)) == 0 && e < N) sf[e * NWARP + wid] = make_float2(h[0], l[0]);
    }
    __syncthreads();
    if (wid == 0) {
        const int grp = lane / NWARP, w = lane % NWARP;
        constexpr int ROUNDS = (N + GROUPS - 1) / GROUPS;
        float2 v[ROUNDS];
#pragma unroll
        for (int r = 0; r < ROUNDS; ++r) {
            const int e = r * GROUPS + grp;
            v[r] = e < N ? sf[e * NWARP + w] : make_float2(0.f, 0.f);
        }
        __syncwarp();
#pragma unroll
        for (int r = 0; r < ROUNDS; ++r) {
            float h = v[r].x, l = v[r].y;
#pragma unroll
            for (int o = NWARP / 2; o > 0; o >>= 1)
                two_sum_acc(h, l, __shfl_xor_sync(0xffffffffu, h, o), __shfl_xor_sync(0xffffffffu, l, o));
            const int e = r * GROUPS + grp;
            if (w == 0 && e < N) sred[e] = (double)h + (double)l;
        }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < N; ++e) out[e] = sred[e];
    __syncthreads();
}

// exp(-lam (x - U)^2) in FP32 with the argument formed in float-float arithmetic from
// FP32 hi + lo pairs of x, U and lam (about 44 significant bits), so that the argument keeps
// its precision where |x - U| is large; the result is expf(hi) * (1 - lo) (|lo| is at most
// an ulp of hi, so the first-order factor is exact to FP32).
__device__ __forceinline__ float exp_gauss_ff(float xh, float xl, float Uh, float Ul, float lh, float ll) {
    const float s = xh - Uh;
    const float bp = s - xh;
    float e = (xh - (s - bp)) + (-Uh - bp);
    e += xl - Ul;
    const float ch = s + e;
    const float cl = e - (ch - s);
    const float p = ch * ch;
    const float pe = fmaf(ch, ch, -p) + 2.f * ch * cl;
    const float q = lh * p;
    const float qe = fmaf(lh, p, -q) + (lh * pe + ll * p);
    return expf(-q) * (1.f - qe);
}

// Asks the bulk-copy engine to bring a global byte range into L2 (cp.async.bulk.prefetch,
// sm_90+; a hint, nothing is written).  The start is rounded down and the end up to 16 bytes;
// the pools carry 256 bytes past their end, so the rounded range stays inside the allocation.
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes) {
    const size_t g = __cvta_generic_to_global(p);
    const size_t a = g & ~(size_t)15;
    const size_t n = (g + bytes - a + 15) & ~(size_t)15;
    if (n == 0 || n > 0xFFFFFFF0u) return;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(a), "r"((unsigned)n) : "memory");
}

// minmod (Flux/Slope.jl:20-24) = ½(sign a + sign b)·min(|a|, |b|) with sign(0) = 0, written as
// selects: for every finite input the same value (the smaller of two positives, the larger of
// two negatives, else +0) with fewer instructions than the sign arithmetic
__device__ __forceinline__ double minmod(double a, double b) {
    return (a > 0.0 && b > 0.0) ? fmin(a, b) : ((a < 0.0 && b < 0.0) ? fmax(a, b) : 0.0);
}
__device__ __forceinline__ float minmod(float a, float b) {
    return (a > 0.f && b > 0.f) ? fminf(a, b) : ((a < 0.f && b < 0.f) ? fmaxf(a, b) : 0.f);
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

}  // namespace kg
