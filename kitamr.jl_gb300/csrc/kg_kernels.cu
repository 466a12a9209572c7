// kg_kernels.cu -- sm_103a kernels of the phase-space step.
//
//   slope_kernel          slope! level pass (Flux/Slope.jl:458-1019)
//   solid_kernel          update_solid_cell!  (Boundary/Immersed_boundary.jl:98-146)
//   wall_kernel           update_solid_neighbor! (Immersed_boundary.jl:367-483)
//   flux_collide_kernel   flux! (gather form of Flux.jl:19-344, CAIDVM.jl, DVM.jl) fused with
//                         iterate!(CAIDVM_Marching | Euler) (Theory/Iterate.jl:96-162)
//   residual_kernel       Σ over cells of the residual_check! terms (Solver/Finalize.jl:5-11)
//
// Layout: f of data d is the column-major nv x ndf block at foff[d] (velocity fastest, the
// memory of VsData.df); sdf of d is the nv x ndf x dim block at foff[d]*dim.  One CTA works
// on one physical cell with threads striding its velocity cells, so every global access to
// f / sdf / velocity metadata is coalesced along the velocity index.
//
// T is the storage type of f / sdf (double: plain form; float: mixed form).  In the mixed
// form the per-velocity arithmetic runs in FP32 while the exponent of the Maxwellian, the
// conserved update, the primitive recovery and the wall-density solve stay in FP64, and
// moment sums use compensated (two-sum) FP32 accumulation before an FP64 block reduction.
#include <cuda_runtime.h>
#include "kg_device.cuh"

namespace kg {

template <typename T> struct Arith { using type = double; };
template <> struct Arith<float> { using type = float; };

// Compensated accumulator: plain FP64 sum for double, Neumaier two-sum for float.
template <typename A> struct Acc {
    A s = 0, c = 0;
    __device__ __forceinline__ void add(A x) {
        A t = s + x;
        if (fabs((double)s) >= fabs((double)x)) c += (s - t) + x; else c += (x - t) + s;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};
template <> struct Acc<double> {
    double s = 0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
};

// velocity metadata in the arithmetic precision (FP32 copies for the mixed form)
template <typename A> __device__ __forceinline__ const A* vel(const Dev& P);
template <> __device__ __forceinline__ const double* vel<double>(const Dev& P) { return P.vu; }
template <> __device__ __forceinline__ const float* vel<float>(const Dev& P) { return P.vuf; }
template <typename A> __device__ __forceinline__ const A* wts(const Dev& P);
template <> __device__ __forceinline__ const double* wts<double>(const Dev& P) { return P.vw; }
template <> __device__ __forceinline__ const float* wts<float>(const Dev& P) { return P.vwf; }
// 2^-(D*(lj-li)) when the source cell is finer (exact power of two), else 1
template <int D, typename A> __device__ __forceinline__ A merge_scale(int li, int lj) {
    return lj > li ? (A)ldexpf(1.0f, -D * (lj - li)) : (A)1;
}

// exp of an FP64 exponent into the arithmetic precision: FP64 for the plain form; for the
// mixed form the FP64 argument is split a = hi + lo (hi = float(a)) and
// exp(a) = expf(hi) * (1 + lo), accurate to FP32 rounding with a handful of FP64 operations
template <typename A> __device__ __forceinline__ A exp_arg(double a);
template <> __device__ __forceinline__ double exp_arg<double>(double a) { return exp(a); }
template <> __device__ __forceinline__ float exp_arg<float>(double a) {
    const float hi = (float)a;
    const float lo = (float)(a - (double)hi);
    return expf(hi) * (1.0f + lo);
}

struct VGridView {
    int64_t goff;
    int nv;
    const double* vu;
    int64_t PG;
    __device__ __forceinline__ double u(int i, int d) const { return vu[(int64_t)d * PG + goff + i]; }
};

__device__ __forceinline__ VGridView grid_view(const Dev& P, int data) {
    VGridView g;
    int gr = P.dgrid[data];
    g.goff = P.g_off[gr];
    g.nv = (int)(P.g_off[gr + 1] - g.goff);
    g.vu = P.vu;
    g.PG = P.PG;
    return g;
}

// =============================================================================
// slope
// =============================================================================
// per-neighbour constants of a slope list (set up once per CTA, one thread per entry): where
// the neighbour's f and sdf live, its velocity count, its pairing rows and velocity levels,
// and the transverse midpoint offsets in the arithmetic precision (0 when not projected)
template <typename A, typename T> struct SlopeNbrA {
    const T* fn;
    const T* sn;
    const int32_t* pj0;    // pairing rows (my grid <- neighbour's grid), when pair >= 0
    const int32_t* pcnt;
    const int8_t* vl;      // the neighbour grid's velocity levels
    A dm[MAXD];
    int32_t nvn, pair, any;
};
constexpr int MAX_SLOPE_NBR = 2 * MAXD * 4;   // 2 sides x dim x 2^(dim-1) neighbours

template <int D, int NDF, typename T>
__device__ __forceinline__ void slope_side(int i, int li, const typename Arith<T>::type* fc,
                                           const SlopeNbrA<typename Arith<T>::type, T>* nb, int cnt,
                                           typename Arith<T>::type inv_ds, typename Arith<T>::type inv_cnt,
                                           typename Arith<T>::type* s) {
    using A = typename Arith<T>::type;
    A acc[NDF];
#pragma unroll
    for (int k = 0; k < NDF; ++k) acc[k] = 0;
    for (int n = 0; n < cnt; ++n) {
        const SlopeNbrA<A, T>& r = nb[n];
        const T* fn = r.fn;
        const T* sn = r.sn;
        const int nvn = r.nvn;
        const bool paired = r.pair >= 0;
        int j0 = i, jc = 1;
        if (paired) { j0 = r.pj0[i]; jc = r.pcnt[i]; }
        for (int j = j0; j < j0 + jc; ++j) {
            const A sc = paired ? merge_scale<D, A>(li, r.vl[j]) : (A)1;
#pragma unroll
            for (int k = 0; k < NDF; ++k) {
                A p = (A)fn[k * nvn + j];
                if (r.any) {
#pragma unroll
                    for (int t = 0; t < D; ++t)
                        if (r.dm[t] != (A)0) p += r.dm[t] * (A)sn[(t * NDF + k) * nvn + j];
                }
                acc[k] += (fc[k] - p) * sc * inv_ds;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NDF; ++k) s[k] = acc[k] * inv_cnt;
}

#ifndef KG_SLOPE_PPT
#define KG_SLOPE_PPT 1
#endif
template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

// neighbours a side of the slope kernel's loads-first path: every side's (2^(D-1)), but one in
// the FP64 3D form, whose registers would cost resident CTAs
template <int D, typename T> constexpr int SLOPE_SIMPLE_MC = (D == 3 && sizeof(T) == 8) ? 1 : 1 << (D - 1);

// NT: threads per CTA (128 for layouts of small velocity grids, whose cells would leave half
// of a 256-thread CTA idle)
// One CTA per work item: a pass cell and a chunk of SLOPE_CHUNK of its velocity cells (every
// velocity cell's slope is independent of the others').
template <int D, int NDF, typename T, int NT>
__global__ void __launch_bounds__(NT) slope_kernel(Dev P, int item_base) {
    using A = typename Arith<T>::type;
    static_assert(SLOPE_CHUNK % (2 * NT) == 0, "a chunk is whole passes of the CTA");
    int pc = item_base + blockIdx.x, v0 = 0;
    if (P.slope_split) {
        pc = P.slope_items[2 * pc];
        v0 = P.slope_items[2 * (item_base + blockIdx.x) + 1] * P.slope_chunk;
    }
    const SlopeCell& SC = P.screc[pc];
    if (SC.regular) {
        // regular cell (one record, no shared-memory setup): in every direction
        // minmod((f - f_A)/ds_A, (f - f_B)/ds_B) -- slope_side with its loops and unit factors
        // resolved.  Several velocity cells per thread and pass: all their loads are issued
        // before any store, so each thread keeps that many sets of loads in flight.
        const int nv = SC.nv;
        const int v1 = P.slope_split ? (int)min((int64_t)nv, (int64_t)v0 + P.slope_chunk) : nv;
        const T* fcell = (const T*)P.f_in + SC.foff;
        T* scell = (T*)P.sdf + SC.foff * D;
        if (threadIdx.x < NDF) prefetch_l2(fcell + (int64_t)threadIdx.x * nv + v0, sizeof(T) * (size_t)(v1 - v0));
        const T* fa[D];
        const T* fb[D];
        A ia[D], ib[D];
#pragma unroll
        for (int dir = 0; dir < D; ++dir) {
            fa[dir] = (const T*)P.f_in + SC.nfoff[2 * dir];
            fb[dir] = (const T*)P.f_in + SC.nfoff[2 * dir + 1];
            if constexpr (sizeof(A) == 4) { ia[dir] = SC.inv_f[2 * dir]; ib[dir] = SC.inv_f[2 * dir + 1]; }
            else { ia[dir] = SC.inv_d[2 * dir]; ib[dir] = SC.inv_d[2 * dir + 1]; }
        }
        // pairs of neighbouring velocity cells per thread and vector loads and stores (8 bytes in
        // the mixed form, 16 in FP64) when every block the cell reads and writes starts at an even
        // element: the cell's and its neighbours' f offsets and its velocity count even (chunks
        // start at multiples of SLOPE_CHUNK); the same arithmetic per velocity cell
        bool pairs = ((SC.foff | (int64_t)nv) & 1) == 0;
#pragma unroll
        for (int q = 0; q < 2 * D; ++q) pairs = pairs && (SC.nfoff[q] & 1) == 0;
        if (pairs) {
            using T2 = typename Vec2<T>::type;
            constexpr int PPT = KG_SLOPE_PPT;   // pairs per thread and pass
            const int q1 = v1 >> 1;
            const T2* fc2[NDF];
            const T2* fa2[D][NDF];
            const T2* fb2[D][NDF];
            T2* sc2[D][NDF];
#pragma unroll
            for (int k = 0; k < NDF; ++k) {
                fc2[k] = reinterpret_cast<const T2*>(fcell + (int64_t)k * nv);
#pragma unroll
                for (int dir = 0; dir < D; ++dir) {
                    fa2[dir][k] = reinterpret_cast<const T2*>(fa[dir] + (int64_t)k * nv);
                    fb2[dir][k] = reinterpret_cast<const T2*>(fb[dir] + (int64_t)k * nv);
                    sc2[dir][k] = reinterpret_cast<T2*>(scell + (int64_t)(dir * NDF + k) * nv);
                }
            }
            for (int q0 = (v0 >> 1) + threadIdx.x; q0 < q1; q0 += PPT * NT) {
                int iq[PPT], jq[PPT];
#pragma unroll
                for (int v = 0; v < PPT; ++v) {
                    iq[v] = q0 + v * NT;
                    jq[v] = iq[v] < q1 ? iq[v] : q0;
                }
                T2 fc[PPT][NDF], a[PPT][D][NDF], b[PPT][D][NDF];
#pragma unroll
                for (int v = 0; v < PPT; ++v) {
#pragma unroll
                    for (int k = 0; k < NDF; ++k) {
                        fc[v][k] = fc2[k][jq[v]];
#pragma unroll
                        for (int dir = 0; dir < D; ++dir) {
                            a[v][dir][k] = fa2[dir][k][jq[v]];
                            b[v][dir][k] = fb2[dir][k][jq[v]];
                        }
                    }
                }
#pragma unroll
                for (int v = 0; v < PPT; ++v) {
                    if (v > 0 && iq[v] >= q1) break;
#pragma unroll
                    for (int dir = 0; dir < D; ++dir) {
#pragma unroll
                        for (int k = 0; k < NDF; ++k) {
                            T2 o;
                            o.x = (T)minmod(((A)fc[v][k].x - (A)a[v][dir][k].x) * ia[dir], ((A)fc[v][k].x - (A)b[v][dir][k].x) * ib[dir]);
                            o.y = (T)minmod(((A)fc[v][k].y - (A)a[v][dir][k].y) * ia[dir], ((A)fc[v][k].y - (A)b[v][dir][k].y) * ib[dir]);
                            sc2[dir][k][iq[v]] = o;
                        }
                    }
                }
            }
            return;
        }
        // velocity cells per thread and pass (measured on the 3D sphere, mixed form: 2 beats 3
        // and 4, whose registers cost resident CTAs)
        constexpr int VPT = 2;
        for (int i0 = v0 + threadIdx.x; i0 < v1; i0 += VPT * NT) {
            int iv[VPT], jv[VPT];
#pragma unroll
            for (int v = 0; v < VPT; ++v) {
                iv[v] = i0 + v * NT;
                jv[v] = iv[v] < v1 ? iv[v] : i0;    // a valid index for the loads
            }
            A fc[VPT][NDF], a[VPT][D][NDF], b[VPT][D][NDF];
#pragma unroll
            for (int v = 0; v < VPT; ++v) {
#pragma unroll
                for (int k = 0; k < NDF; ++k) fc[v][k] = (A)fcell[k * nv + jv[v]];
#pragma unroll
                for (int dir = 0; dir < D; ++dir) {
#pragma unroll
                    for (int k = 0; k < NDF; ++k) {
                        a[v][dir][k] = (A)fa[dir][k * nv + jv[v]];
                        b[v][dir][k] = (A)fb[dir][k * nv + jv[v]];
                    }
                }
            }
#pragma unroll
            for (int v = 0; v < VPT; ++v) {
                if (v > 0 && iv[v] >= v1) break;
#pragma unroll
                for (int dir = 0; dir < D; ++dir) {
#pragma unroll
                    for (int k = 0; k < NDF; ++k)
                        scell[(dir * NDF + k) * nv + iv[v]] =
                            (T)minmod((fc[v][k] - a[v][dir][k]) * ia[dir], (fc[v][k] - b[v][dir][k]) * ib[dir]);
                }
            }
        }
        return;
    }
    const int cell = P.pass_cells[pc];
    const int op0 = P.cell_slope_op[pc];
    const VGridView g = grid_view(P, cell);
    const int nv = g.nv;
    const int64_t fo = P.foff[cell];
    const T* fcell = (const T*)P.f_in + fo;
    T* scell = (T*)P.sdf + fo * D;
    __shared__ SlopeOp ops[MAXD];
    __shared__ SlopeNbrA<A, T> snb[MAX_SLOPE_NBR];
    __shared__ int sbase[2 * MAXD + 1];
    __shared__ A sconst[4 * MAXD];   // inv_dsA, inv_dsB, 1/cntA, 1/cntB per direction
    __shared__ int ssimple;          // every neighbour on the cell's own grid
    if (threadIdx.x < D) ops[threadIdx.x] = P.slope_ops[op0 + threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
        int n = 0, simple = 1;
        for (int dir = 0; dir < D; ++dir) {
            const SlopeOp& op = ops[dir];
            for (int side = 0; side < 2; ++side) {
                const int cnt = (op.kind == SLOPE_ONE || op.kind == SLOPE_TWO) ? (side == 0 ? op.cntA : (op.kind == SLOPE_TWO ? op.cntB : 0)) : 0;
                sbase[2 * dir + side] = n;
                n += cnt;
                for (int e = 0; e < cnt; ++e)
                    if (e >= SLOPE_SIMPLE_MC<D, T> || P.slope_nbr[(side == 0 ? op.listA : op.listB) + e].pair >= 0) simple = 0;
            }
            sconst[4 * dir + 0] = (A)op.inv_dsA;
            sconst[4 * dir + 1] = (A)op.inv_dsB;
            sconst[4 * dir + 2] = op.cntA > 0 ? (A)1 / (A)op.cntA : (A)0;
            sconst[4 * dir + 3] = op.cntB > 0 ? (A)1 / (A)op.cntB : (A)0;
        }
        sbase[2 * D] = n < MAX_SLOPE_NBR ? n : MAX_SLOPE_NBR;
        ssimple = simple;
    }
    __syncthreads();
    // one thread per neighbour entry (at most 2 * dim * 2^(dim-1), checked on the host)
    if (threadIdx.x < sbase[2 * D]) {
        const int e = threadIdx.x;
        int ds = 0;
        while (ds + 1 < 2 * D && sbase[ds + 1] <= e) ++ds;
        const int dir = ds >> 1, side = ds & 1;
        const SlopeOp& op = ops[dir];
        const NbrRef r = P.slope_nbr[(side == 0 ? op.listA : op.listB) + (e - sbase[ds])];
        const bool proj = side == 0 ? op.projA : op.projB;
        const double* cm = P.dmid + (int64_t)cell * MAXD;
        const double* nm = P.dmid + (int64_t)r.data * MAXD;
        SlopeNbrA<A, T> c;
        const int64_t nfo = P.foff[r.data];
        c.fn = (const T*)P.f_in + nfo;
        c.sn = (const T*)P.sdf + nfo * D;
        c.nvn = P.dnv[r.data];
        c.pair = r.pair;
        const int64_t gn = P.g_off[P.dgrid[r.data]];
        c.vl = P.vlev + gn;
        if (r.pair >= 0) {
            const int64_t po = P.p_off[r.pair];
            c.pj0 = P.p_j0 + po;
            c.pcnt = P.p_cnt + po;
        } else {
            c.pj0 = nullptr;
            c.pcnt = nullptr;
        }
        c.any = 0;
#pragma unroll
        for (int t = 0; t < MAXD; ++t) {
            c.dm[t] = (t < D && proj && t != dir) ? (A)(cm[t] - nm[t]) : (A)0;
            c.any |= c.dm[t] != (A)0;
        }
        snb[e] = c;
    }
    __syncthreads();
    const int v1 = P.slope_split ? (int)min((int64_t)nv, (int64_t)v0 + P.slope_chunk) : nv;
    if (ssimple) {
        // every neighbour on the cell's own grid (the cells beside a coarser one, whose side
        // projects that neighbour with its transverse slopes, those beside finer ones, and the
        // cells at domain boundaries): slope_side's arithmetic for unpaired entries, in its
        // order, with every entry's loads issued before any is used
        constexpr int MC = SLOPE_SIMPLE_MC<D, T>;
        for (int i = v0 + threadIdx.x; i < v1; i += NT) {
            A fc[NDF];
#pragma unroll
            for (int k = 0; k < NDF; ++k) fc[k] = (A)fcell[k * nv + i];
            A pv[D][2][MC][NDF];
#pragma unroll
            for (int dir = 0; dir < D; ++dir) {
#pragma unroll
                for (int side = 0; side < 2; ++side) {
                    const int cnt = (ops[dir].kind == SLOPE_ONE || ops[dir].kind == SLOPE_TWO)
                                  ? (side == 0 ? ops[dir].cntA : (ops[dir].kind == SLOPE_TWO ? ops[dir].cntB : 0)) : 0;
#pragma unroll
                    for (int e = 0; e < MC; ++e) {
                        const SlopeNbrA<A, T>& r = snb[sbase[2 * dir + side] + (e < cnt ? e : 0)];
#pragma unroll
                        for (int k = 0; k < NDF; ++k) {
                            A p = 0;
                            if (e < cnt) {
                                p = (A)r.fn[k * r.nvn + i];
                                if (r.any) {
#pragma unroll
                                    for (int t = 0; t < D; ++t)
                                        if (r.dm[t] != (A)0) p += r.dm[t] * (A)r.sn[(t * NDF + k) * r.nvn + i];
                                }
                            }
                            pv[dir][side][e][k] = p;
                        }
                    }
                }
            }
#pragma unroll
            for (int dir = 0; dir < D; ++dir) {
                const SlopeOp& op = ops[dir];
                if (op.kind == SLOPE_SKIP) continue;
                A out[NDF];
                if (op.kind == SLOPE_ZERO) {
#pragma unroll
                    for (int k = 0; k < NDF; ++k) out[k] = 0;
                } else {
                    const int cA = op.cntA, cB = op.kind == SLOPE_TWO ? op.cntB : 0;
#pragma unroll
                    for (int k = 0; k < NDF; ++k) {
                        A accA = 0, accB = 0;
#pragma unroll
                        for (int e = 0; e < MC; ++e)
                            if (e < cA) accA += (fc[k] - pv[dir][0][e][k]) * (A)1 * sconst[4 * dir];
                        const A sA = accA * sconst[4 * dir + 2];
                        if (op.kind == SLOPE_ONE) {
                            out[k] = sA;
                        } else {
#pragma unroll
                            for (int e = 0; e < MC; ++e)
                                if (e < cB) accB += (fc[k] - pv[dir][1][e][k]) * (A)1 * sconst[4 * dir + 1];
                            out[k] = minmod(sA, accB * sconst[4 * dir + 3]);
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < NDF; ++k) scell[(dir * NDF + k) * nv + i] = (T)out[k];
            }
        }
        return;
    }
    for (int i = v0 + threadIdx.x; i < v1; i += NT) {
        const int li = P.vlev[g.goff + i];
        A fc[NDF];
#pragma unroll
        for (int k = 0; k < NDF; ++k) fc[k] = (A)fcell[k * nv + i];
#pragma unroll
        for (int dir = 0; dir < D; ++dir) {
            const SlopeOp& op = ops[dir];
            if (op.kind == SLOPE_SKIP) continue;
            A out[NDF];
            if (op.kind == SLOPE_ZERO) {
#pragma unroll
                for (int k = 0; k < NDF; ++k) out[k] = 0;
            } else {
                A sA[NDF];
                slope_side<D, NDF, T>(i, li, fc, &snb[sbase[2 * dir]], op.cntA, sconst[4 * dir], sconst[4 * dir + 2], sA);
                if (op.kind == SLOPE_ONE) {
#pragma unroll
                    for (int k = 0; k < NDF; ++k) out[k] = sA[k];
                } else {
                    A sB[NDF];
                    slope_side<D, NDF, T>(i, li, fc, &snb[sbase[2 * dir + 1]], op.cntB, sconst[4 * dir + 1], sconst[4 * dir + 3], sB);
#pragma unroll
                    for (int k = 0; k < NDF; ++k) out[k] = minmod(sA[k], sB[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < NDF; ++k) scell[(dir * NDF + k) * nv + i] = (T)out[k];
        }
    }
}

// Compensated (Kahan) accumulator for the FP32 arithmetic of the mixed form; plain sum in FP64.
template <typename A> struct KSum {
    A s = 0, c = 0;
    __device__ __forceinline__ void add(A x) { A y = x - c; A t = s + y; c = (t - s) - y; s = t; }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <> struct KSum<double> {
    double s = 0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
};

// Block sum of compensated per-thread accumulators into FP64 results (NT: threads of the block).
template <int N, int NT = BLOCK>
__device__ __forceinline__ void block_sum_ks(const KSum<double> (&v)[N], double (&out)[N], double* sred) {
#pragma unroll
    for (int e = 0; e < N; ++e) out[e] = v[e].s;
    block_sum<N, NT>(out, sred);
}
template <int N, int NT = BLOCK>
__device__ __forceinline__ void block_sum_ks(const KSum<float> (&v)[N], double (&out)[N], double* sred) {
    float hi[N], lo[N];
#pragma unroll
    for (int e = 0; e < N; ++e) { hi[e] = v[e].s; lo[e] = -v[e].c; }
    block_sum_ff<N, NT>(hi, lo, out, sred);
}

// limiter ratio: exact division in FP64; the fast FP32 division (2 ulp) in the mixed form,
// where it only scales the slope term through min(|ratio|, 1)
__device__ __forceinline__ double lim_div(double a, double b) { return a / b; }
__device__ __forceinline__ float lim_div(float a, float b) { return __fdividef(a, b); }

// =============================================================================
// immersed boundary
// =============================================================================
// Per-CTA constants of one image_df / update_solid_cell! source list, in the arithmetic
// precision: the unit direction l/|l| and the offset l of each source, and where its f lives.
template <typename A> struct IbNbrA {
    A lhat[MAXD];
    A dx[MAXD];
    int64_t fo, gn;
    int32_t nvn, pair;
};
constexpr int MAX_IB_NBR = 2 * MAXD + 1;   // face neighbours + the donor (checked by construction)

// filled by the first `cnt` threads; the caller synchronises before use
template <int D, typename A>
__device__ __forceinline__ void ib_setup(const Dev& P, int list, int cnt, IbNbrA<A>* nb) {
    const int n = threadIdx.x;
    if (n >= cnt || n >= MAX_IB_NBR) return;
    const double* dx = P.ib_dx + (int64_t)(list + n) * MAXD;
    const NbrRef r = P.ib_nbr[list + n];
    A l[D], nl = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) { l[d] = (A)dx[d]; nl += l[d] * l[d]; }
    nl = sqrt(nl);
    IbNbrA<A> c;
#pragma unroll
    for (int d = 0; d < MAXD; ++d) { c.lhat[d] = d < D ? l[d] / nl : (A)0; c.dx[d] = d < D ? l[d] : (A)0; }
    c.fo = P.foff[r.data];
    c.nvn = P.dnv[r.data];
    c.pair = r.pair;
    c.gn = r.pair >= 0 ? P.g_off[P.dgrid[r.data]] : 0;
    nb[n] = c;
}

// Σ_n weight_n(u) * merge_n(f_n + sdf_n . dx_n) over a source list, for target velocity i
// (vs_extrapolate! with the directional weights of update_solid_cell! / image_df).
template <int D, int NDF, typename T>
__device__ __forceinline__ void extrapolate(const Dev& P, const VGridView& g, int i, int li,
                                            const IbNbrA<typename Arith<T>::type>* nb, int cnt,
                                            typename Arith<T>::type* out) {
    using A = typename Arith<T>::type;
    const T* f = (const T*)P.f_in;
    const T* sdf = (const T*)P.sdf;
    const A* VU = vel<A>(P);
    A u[D], un = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) { u[d] = VU[(int64_t)d * P.PG + g.goff + i]; un += u[d] * u[d]; }
    un = sqrt(un);
    A W[MAX_IB_NBR];
    A wsum = 0;
    for (int n = 0; n < cnt; ++n) {
        A ul = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) ul += u[d] * nb[n].lhat[d];
        A v = ul / un;
        v = v > (A)0 ? v : (A)0;
        W[n] = v * v;
        wsum += W[n];
    }
#pragma unroll
    for (int k = 0; k < NDF; ++k) out[k] = 0;
    for (int n = 0; n < cnt; ++n) {
        const A wi = wsum == (A)0 ? (A)1 / (A)cnt : W[n] / wsum;
        const IbNbrA<A>& r = nb[n];
        const int nvn = r.nvn;
        const T* fn = f + r.fo;
        const T* sn = sdf + r.fo * D;
        int j0 = i, jc = 1;
        if (r.pair >= 0) {
            const int64_t po = P.p_off[r.pair] + i;
            j0 = P.p_j0[po];
            jc = P.p_cnt[po];
        }
        for (int j = j0; j < j0 + jc; ++j) {
            const A sc = r.pair >= 0 ? merge_scale<D, A>(li, P.vlev[r.gn + j]) : (A)1;
#pragma unroll
            for (int k = 0; k < NDF; ++k) {
                A v = (A)fn[k * nvn + j];
                A sv = 0;
#pragma unroll
                for (int d = 0; d < D; ++d) sv += (A)sn[(d * NDF + k) * nvn + j] * r.dx[d];
                out[k] += (v + sv) * sc * wi;
            }
        }
    }
}

// moments of one velocity cell into compensated accumulators in the arithmetic precision
template <int D, int NDF, typename A>
__device__ __forceinline__ void moments_add_a(const A* u, const A wgt, const A* fv, KSum<A>* m) {
    A u2 = 0;
    m[0].add(wgt * fv[0]);
#pragma unroll
    for (int d = 0; d < D; ++d) { m[1 + d].add(wgt * u[d] * fv[0]); u2 += u[d] * u[d]; }
    if (NDF == 2) m[D + 1].add((A)0.5 * wgt * (u2 * fv[0] + fv[NDF - 1]));
    else m[D + 1].add((A)0.5 * wgt * u2 * fv[0]);
}

// update_solid_cell! (Immersed_boundary.jl:98-146): a solid ghost cell's f is extrapolated
// from its fluid neighbours; its w and prim are the moments of that f.
template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK) solid_kernel(Dev P) {
    using A = typename Arith<T>::type;
    __shared__ double sred[(D + 2) * (BLOCK / 32)];
    __shared__ IbNbrA<A> snb[MAX_IB_NBR];
    const SolidOp op = P.solid_ops[blockIdx.x];
    ib_setup<D, A>(P, op.list, op.cnt, snb);
    __syncthreads();
    const VGridView g = grid_view(P, op.cell);
    const int nv = g.nv;
    const int64_t fo = P.foff[op.cell];
    T* fa = (T*)P.f_in + fo;
    T* fb = (T*)P.f_out + fo;
    const A* VU = vel<A>(P);
    const A* VW = wts<A>(P) + g.goff;
    KSum<A> m[D + 2];
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        const int li = P.vlev[g.goff + i];
        A va[NDF];
        extrapolate<D, NDF, T>(P, g, i, li, snb, op.cnt, va);
#pragma unroll
        for (int k = 0; k < NDF; ++k) { fa[(int64_t)k * nv + i] = (T)va[k]; fb[(int64_t)k * nv + i] = (T)va[k]; }
        A u[D];
#pragma unroll
        for (int d = 0; d < D; ++d) u[d] = VU[(int64_t)d * P.PG + g.goff + i];
        moments_add_a<D, NDF, A>(u, VW[i], va, m);
    }
    double mw[D + 2];
    block_sum_ks<D + 2>(m, mw, sred);
    if (threadIdx.x == 0) {
        double* w = P.w + (int64_t)op.cell * MAXW;
        double* pr = P.prim + (int64_t)op.cell * MAXW;
#pragma unroll
        for (int e = 0; e < D + 2; ++e) w[e] = mw[e];
        get_prim<D>(mw, P.probs[P.dprob[op.cell]].gamma, pr);
    }
}

// shared memory of wall_kernel for a donor grid of nv velocity cells: the wall Maxwellian's
// factor tables and the direction flag per velocity (the image extrapolation waits in the
// wall record's output f block, so a 24^3 grid still leaves room for 4 CTAs per SM)
template <int D, int NDF, typename A>
__host__ __device__ __forceinline__ size_t wall_smem(int nv, int max_axis) {
    return (size_t)D * max_axis * sizeof(A) + (size_t)nv;
}

// update_solid_neighbor! (Immersed_boundary.jl:367-483): the SolidNeighbor's f is the
// diffuse-wall Maxwellian (density from the zero-mass-flux condition) for velocities leaving
// the wall and the slope-limited image extrapolation for velocities entering it, blended on
// the cut velocity cells; the wall-direction slope is kept for the flux of the donor.
template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK) wall_kernel(Dev P) {
    using A = typename Arith<T>::type;
    extern __shared__ __align__(16) unsigned char wsh[];
    __shared__ double sred[2 * (BLOCK / 32)];
    __shared__ IbNbrA<A> snb[MAX_IB_NBR];
    // per-CTA constants in the arithmetic precision, set by thread 0
    enum { W_N = 0, W_IDXS = W_N + MAXD, W_IDXF, W_DXL, W_PRE, W_BK, W_COUNT };
    __shared__ A wc[W_COUNT];
    const WallOp op = P.wall_ops[blockIdx.x];
    const VGridView g = grid_view(P, op.donor);
    const VGridView gs = grid_view(P, op.solid);
    const int nv = g.nv, nvs = gs.nv;
    const int gid = P.dgrid[op.donor];
    const int MA = P.max_axis;
    A* Ew = (A*)wsh;                                 // D * max_axis: 1D factors of the wall Maxwellian
    unsigned char* out_dir = (unsigned char*)(Ew + (size_t)D * MA);   // nv: u.n >= 0
    // the record's two f blocks: wa ends with the new f; wb holds the image extrapolation
    // (aux) until the last pass copies wa over it
    T* wa = (T*)P.f_in + P.foff[op.data];
    T* wb = (T*)P.f_out + P.foff[op.data];
    ib_setup<D, A>(P, op.list, op.cnt, snb);
    const double lam = op.bc[D + 1];
    const double Kw = P.probs[P.dprob[op.donor]].K;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int d = 0; d < MAXD; ++d) wc[W_N + d] = (A)op.normal[d];
        wc[W_IDXS] = (A)(1.0 / op.dxs);
        wc[W_IDXF] = (A)(1.0 / op.dxf);
        wc[W_DXL] = (A)op.dxL;
        wc[W_PRE] = (A)(D == 2 ? lam / PI : pow(lam / PI, 1.5));
        wc[W_BK] = (A)(Kw / (2.0 * lam));
    }
    // 1D factors exp(-lam (x - U_d)^2) of the wall Maxwellian at the grid's axis coordinates
    // (FP64 exponents; discrete_maxwell_2D2F / 3D1F)
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const int a0 = P.ax_off[gid * MAXD + d], na = P.ax_off[gid * MAXD + d + 1] - a0;
        for (int a = threadIdx.x; a < na; a += BLOCK) {
            const double cu = P.ax_val[a0 + a] - op.bc[1 + d];
            Ew[d * MA + a] = exp_arg<A>(-lam * cu * cu);
        }
    }
    __syncthreads();
    const T* fc = (const T*)P.f_in + P.foff[op.donor];
    const T* fsol = (const T*)P.f_in + P.foff[op.solid];
    const int64_t wo = P.foff[op.data];
    T* wsdf = (T*)P.sdf + wo * D;
    const double* cvcw = P.cvcw + op.cvcw_off;
    const int dir = op.dir;
    const A* VU = vel<A>(P);
    const uint16_t* vx = P.vidx + g.goff;
    const A idxs = wc[W_IDXS], idxf = wc[W_IDXF], dxL = wc[W_DXL], pre = wc[W_PRE];
    // the wall Maxwellian with rho = 1 at velocity i, from its factor tables
    auto mh_of = [&](int i) {
        A m = pre;
#pragma unroll
        for (int d = 0; d < D; ++d) m *= Ew[d * MA + vx[(int64_t)d * P.PG + i]];
        return m;
    };
    KSum<A> red[2];   // MuR, SF
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        const int li = P.vlev[g.goff + i];
        // the sign of u.n picks the branch: FP64, as in the reference
        double vnd = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) vnd += g.u(i, d) * op.normal[d];
        const bool leaving = vnd >= 0.0;
        out_dir[i] = leaving;
        const A vn = (A)vnd;
        A ib[NDF];
        extrapolate<D, NDF, T>(P, g, i, li, snb, op.cnt, ib);
        // boundary_slope! (Immersed_boundary.jl:396-435)
        A sL[NDF];
        int j0 = i, jc = 1;
        if (op.spair >= 0) {
            const int64_t po = P.p_off[op.spair] + i;
            j0 = P.p_j0[po];
            jc = P.p_cnt[po];
        }
#pragma unroll
        for (int k = 0; k < NDF; ++k) sL[k] = 0;
        for (int j = j0; j < j0 + jc; ++j) {
            const A sc = op.spair >= 0 ? merge_scale<D, A>(li, P.vlev[gs.goff + j]) : (A)1;
#pragma unroll
            for (int k = 0; k < NDF; ++k)
                sL[k] += ((A)fc[(int64_t)k * nv + i] - (A)fsol[(int64_t)k * nvs + j]) * sc * idxs;
        }
        A a0 = 0;
#pragma unroll
        for (int k = 0; k < NDF; ++k) {
            const A fck = (A)fc[(int64_t)k * nv + i];
            A ss = minmod(sL[k], (ib[k] - fck) * idxf);
            const A r = fabs(lim_div(ib[k] - (A)JL_EPS, ss * dxL + (A)JL_EPS));
            ss = (r < (A)1 ? r : (A)1) * ss;
            wsdf[((int64_t)dir * NDF + k) * nv + i] = (T)ss;
            const A a = ib[k] + ss * dxL;
            wb[(int64_t)k * nv + i] = (T)a;
            if (k == 0) a0 = a;
        }
        const A mh = mh_of(i);
        const A cw = (A)cvcw[i];
        if (leaving) red[0].add(cw * vn * mh);
        else red[1].add(cw * vn * a0);
    }
    __syncthreads();
    for (int a = threadIdx.x; a < op.cut_cnt; a += BLOCK) {
        const int idx = P.cut_idx[op.cut_off + a];
        A vn = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) vn += VU[(int64_t)d * P.PG + g.goff + idx] * wc[W_N + d];
        red[0].add((A)P.cut_sw[op.cut_off + a] * vn * mh_of(idx));
        red[1].add((A)P.cut_gw[op.cut_off + a] * vn * (A)wb[idx]);
    }
    double rs[2];
    block_sum_ks<2>(red, rs, sred);
    const double rho_w = -rs[1] / rs[0];
    const A rw = (A)rho_w, bk = wc[W_BK];
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        A v[NDF];
        if (out_dir[i]) {
            const A mh = mh_of(i);
            v[0] = mh * rw;
            if (NDF == 2) v[NDF - 1] = mh * bk * rw;
        } else {
#pragma unroll
            for (int k = 0; k < NDF; ++k) v[k] = (A)wb[(int64_t)k * nv + i];
        }
#pragma unroll
        for (int k = 0; k < NDF; ++k) wa[(int64_t)k * nv + i] = (T)v[k];
    }
    __syncthreads();
    for (int a = threadIdx.x; a < op.cut_cnt; a += BLOCK) {
        const int idx = P.cut_idx[op.cut_off + a];
        const A gw = (A)P.cut_gw[op.cut_off + a], sw = (A)P.cut_sw[op.cut_off + a];
        const A mh = mh_of(idx);
        A mv[NDF];
        mv[0] = mh * rw;
        if (NDF == 2) mv[NDF - 1] = mh * bk * rw;
#pragma unroll
        for (int k = 0; k < NDF; ++k)
            wa[(int64_t)k * nv + idx] = (T)((gw * (A)wb[(int64_t)k * nv + idx] + sw * mv[k]) / (gw + sw));
    }
    __syncthreads();
    // both buffers carry the record's f (the next step reads the other one)
    for (int64_t e = threadIdx.x; e < (int64_t)NDF * nv; e += BLOCK) wb[e] = wa[e];
}

// =============================================================================
// flux + collision
// =============================================================================
template <int D, typename A>
__device__ __forceinline__ A pp_recon(A f, const A* s, const double* ds, const A* dx) {
    // positivity_preserving_reconstruct (Flux/CAIDVM.jl:127-142)
    A sabs = 0, sdx = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) sabs += (A)ds[d] * fabs(s[d]);
#pragma unroll
    for (int d = 0; d < D; ++d) sdx += dx[d] * s[d];
    A th = fabs((f - (A)JL_EPS) / ((A)0.5 * sabs + (A)EPS_REF));
    th = th < (A)1 ? th : (A)1;
    return f + th * sdx;
}
template <int D, typename A>
__device__ __forceinline__ A plain_recon(A f, const A* s, const A* dx) {
    A sdx = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) sdx += dx[d] * s[d];
    return f + sdx;
}

// micro flux leaving data `dat` (velocity j of grid gv) through a face; mode 0 = positivity
// reconstruction, 1 = plain reconstruction, 2 = unreconstructed
template <int D, int NDF, typename T>
__device__ __forceinline__ void side_micro(const Dev& P, int dat, int64_t fo, int nvd, const VGridView& gv, int j,
                                           const double* fmid, const double* cmid, const double* ds, double dt, int dir,
                                           int mode, typename Arith<T>::type* out) {
    using A = typename Arith<T>::type;
    const T* f = (const T*)P.f_in + fo;
    const T* sdf = (const T*)P.sdf + fo * D;
    A dx[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dx[d] = (A)(fmid[d] - gv.u(j, d) * dt - cmid[d]);
    const A vn = (A)gv.u(j, dir);
#pragma unroll
    for (int k = 0; k < NDF; ++k) {
        A fk = (A)f[(int64_t)k * nvd + j];
        if (mode == 2) { out[k] = fk * vn; continue; }
        A s[D];
#pragma unroll
        for (int d = 0; d < D; ++d) s[d] = (A)sdf[((int64_t)d * NDF + k) * nvd + j];
        out[k] = (mode == 0 ? pp_recon<D, A>(fk, s, ds, dx) : plain_recon<D, A>(fk, s, dx)) * vn;
    }
}

template <int D, int NDF>
__device__ __forceinline__ void psi_add(double* m, double wgt, const double* u, const double* v) {
    // weight * ψ * micro, ψ = (1, u, |u|²/2 with b) as in micro_to_macro_*
    double u2 = 0.0;
    m[0] += wgt * v[0];
#pragma unroll
    for (int d = 0; d < D; ++d) { m[1 + d] += wgt * u[d] * v[0]; u2 += u[d] * u[d]; }
    if (NDF == 2) m[D + 1] += 0.5 * wgt * (u2 * v[0] + v[NDF - 1]);
    else m[D + 1] += 0.5 * wgt * u2 * v[0];
}

// own-side reconstruction from registers (positivity / plain / none)
template <int D, typename A>
__device__ __forceinline__ A own_recon(int mode, A f, const A* s, const A* dx, const A* ds) {
    if (mode == 2) return f;
    A sdx = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) sdx += dx[d] * s[d];
    if (mode == 1) return f + sdx;
    // positivity_preserving_reconstruct (Flux/CAIDVM.jl:127-142)
    A sabs = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) sabs += ds[d] * fabs(s[d]);
    A th = fabs(lim_div(f - (A)JL_EPS, (A)0.5 * sabs + (A)EPS_REF));
    th = th < (A)1 ? th : (A)1;
    return f + th * sdx;
}

// micro flux of another data item (velocity j of its grid, velocities u) through a face
template <int D, int NDF, typename T, typename A>
__device__ __forceinline__ void other_micro(const T* f, const T* sdf, int nvd, int j, const A* u, const A* dxo,
                                            const A* ds, A adt, int dir, int mode, A* out) {
    A dx[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dx[d] = dxo[d] - u[d] * adt;
    const A ud = D == 2 ? (dir == 0 ? u[0] : u[D - 1]) : (dir == 0 ? u[0] : (dir == 1 ? u[1] : u[D - 1]));
#pragma unroll
    for (int k = 0; k < NDF; ++k) {
        A s[D];
        const A fk = (A)f[k * nvd + j];
        if (mode != 2) {
#pragma unroll
            for (int d = 0; d < D; ++d) s[d] = (A)sdf[(d * NDF + k) * nvd + j];
        }
        out[k] = own_recon<D, A>(mode, fk, s, dx, ds) * ud;
    }
}

// per-incidence constants in the arithmetic precision
template <typename A, typename T> struct IncA {
    A dxm[MAXD];    // face midpoint - my reconstruction centre
    A dxo[MAXD];    // face midpoint - other side's reconstruction centre
    A ods[MAXD];    // other side's ds
    A orient, sarea;
    const T* of;    // other side's f and sdf blocks (inner / solid faces)
    const T* os;
    int32_t onv, pair, ogo;
    int8_t kind, dir, bc_kind, mode_out, mode_in;
};

// Factor tables E[d][a] = exp(-lam (x_a - U_d)^2) of a Maxwellian at the distinct axis
// coordinates x_a of grid gid (exp(-lam|u-U|^2) = Π_d E[d][axis index of u_d]); every thread
// of the block takes entries.  FP64 form: FP64 exponents.
template <int D, int NT = BLOCK>
__device__ __forceinline__ void gauss_table(const Dev& P, int gid, const double* U, double lam, double* E) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const int a0 = P.ax_off[gid * MAXD + d], na = P.ax_off[gid * MAXD + d + 1] - a0;
        for (int a = threadIdx.x; a < na; a += NT) {
            const double cu = P.ax_val[a0 + a] - U[d];
            E[d * P.max_axis + a] = exp(-lam * cu * cu);
        }
    }
}
// Mixed form: FP32 tables whose exponents are formed in float-float arithmetic from the
// FP32 hi + lo pairs of x, U and lam, so no FP64 instruction runs per entry.
// (entry a of axis d at E[(d * max_axis + a) * TS]: TS = 4 for the packed kernel's interleaved
// table of (M_c, M_n, u) factors)
// CW (TS = 4, the collision Maxwellian's table): the peculiar velocity c_d = (u_d - U_hi) - U_lo
// of each axis entry goes to the record's fourth float, so the per-velocity passes read it
template <int D, int NT = BLOCK, int TS = 1, bool CW = false>
__device__ __forceinline__ void gauss_table(const Dev& P, int gid, const float* Uh, const float* Ul, float lh,
                                            float ll, float* E) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const int a0 = P.ax_off[gid * MAXD + d], na = P.ax_off[gid * MAXD + d + 1] - a0;
        for (int a = threadIdx.x; a < na; a += NT) {
            E[(d * P.max_axis + a) * TS] = exp_gauss_ff(P.ax_hi[a0 + a], P.ax_lo[a0 + a], Uh[d], Ul[d], lh, ll);
            if constexpr (CW) E[(d * P.max_axis + a) * TS + 3] = (P.ax_hi[a0 + a] - Uh[d]) - Ul[d];
        }
    }
}

// get_prim_2D / 3D (lib/KitCore/2D.jl:9-16, 3D.jl:12-20) with one reciprocal of ρ and one
// division for λ (the FP64 divisions of the scalar section are its slowest instructions)
template <int D>
__device__ __forceinline__ void get_prim_r(const double* w, double gamma, double* prim) {
    const double inv = 1.0 / w[0];
    prim[0] = w[0];
    double m2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) { prim[1 + d] = w[1 + d] * inv; m2 += w[1 + d] * w[1 + d]; }
    prim[D + 1] = 0.5 * w[0] / ((gamma - 1.0) * (w[D + 1] - 0.5 * m2 * inv));
}

// dynamic shared memory of the flux kernel: convected f (unless it is staged in the cell's
// output block), then the factor tables (two collision Maxwellians, or one per
// Maxwellian-state domain face earlier in the step)
// the packed kernel's dynamic shared memory: the convected (h, b) pairs, then (16-byte
// aligned) the interleaved axis table of D * max_axis float4
__host__ __device__ __forceinline__ size_t packed_table_off(int nv) { return ((size_t)8 * nv + 15) / 16 * 16; }
__host__ __device__ __forceinline__ size_t packed_smem(int max_nv, int max_axis) {
    return packed_table_off(max_nv) + (size_t)16 * 2 * max_axis;
}
template <int D, int NDF, typename A>
__host__ __device__ __forceinline__ size_t flux_smem(int max_nv, int max_axis, int max_bcm, int fst_global) {
    return ((fst_global ? (size_t)0 : (size_t)NDF * max_nv) + (size_t)(max_bcm > 2 ? max_bcm : 2) * D * max_axis) * sizeof(A);
}

// Julia's min of two floats (NaN if either is NaN)
__device__ __forceinline__ double jl_min(double a, double b) { return (a != a || b != b) ? (a + b) : (a < b ? a : b); }

// positivity_preserving_ib! (Boundary/Positivity.jl:13-27): the micro flux a SolidNeighbor's
// reconstruction perturbance sends into the donor through incidence ia at velocity i (which
// enters from the wall): (ndf + ndx . sdf) u_dir area, with ndf = ssdf (x_solid - x_aux)[dir]
// (pert), ndx = face midpoint - u dt - x_solid and sdf the record's slopes (zero but for the
// wall direction, ssdf).
template <int D, int NDF, typename T, typename A, typename IA>
__device__ __forceinline__ void pp_ib_micro(const IA& ia, A pert, int i, const A* u, A adt, A* out) {
    const int dir = ia.dir;
    const A ud = D == 2 ? (dir == 0 ? u[0] : u[D - 1]) : (dir == 0 ? u[0] : (dir == 1 ? u[1] : u[D - 1]));
    const int nv = ia.onv;
#pragma unroll
    for (int k = 0; k < NDF; ++k) {
        A dot = 0, ss = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const A sd = (A)ia.os[(d * NDF + k) * nv + i];
            dot += (ia.dxo[d] - u[d] * adt) * sd;
            if (d == dir) ss = sd;
        }
        out[k] = (ss * pert + dot) * ud * ia.sarea;
    }
}

// The two passes of positivity_preserving_ib! over a donor cell's velocities (kept out of
// line: only donor cells under CIP marching run them).  fst == nullptr: the moments of the
// SolidNeighbors' perturbance micro fluxes into wev (a block reduction); otherwise
// fst += scale * micro (scale = dt / V * theta) at every velocity entering from a wall.
template <int D, int NDF, typename T, int NT>
__device__ __noinline__ void pp_ib_pass(const Incidence* sinc, const IncA<typename Arith<T>::type, T>* sia, int ninc,
                                        int nv, const typename Arith<T>::type* vu, int64_t PG,
                                        const typename Arith<T>::type* vw, typename Arith<T>::type adt,
                                        typename Arith<T>::type scale, typename Arith<T>::type* fst, double* wev,
                                        double* sred) {
    using A = typename Arith<T>::type;
    KSum<A> wpp[D + 2];
    for (int i = threadIdx.x; i < nv; i += NT) {
        A u[D], uu = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) { u[d] = vu[(int64_t)d * PG + i]; uu += u[d] * u[d]; }
        const A wv = vw[i];
        for (int e = 0; e < ninc; ++e) {
            if (!sinc[e].wallrec) continue;
            const IncA<A, T>& ia = sia[e];
            const int dir = ia.dir;
            const A ud = D == 2 ? (dir == 0 ? u[0] : u[D - 1]) : (dir == 0 ? u[0] : (dir == 1 ? u[1] : u[D - 1]));
            if (!(ia.orient * ud > (A)0)) continue;
            A mp[NDF];
            const A pert = sizeof(A) == 4 ? (A)sinc[e].pert_f : (A)sinc[e].pert;
            pp_ib_micro<D, NDF, T, A>(ia, pert, i, u, adt, mp);
            if (fst) {
#pragma unroll
                for (int k = 0; k < NDF; ++k) fst[(int64_t)k * nv + i] += scale * mp[k];
            } else {
                const A b0 = wv * mp[0];
                wpp[0].add(b0);
#pragma unroll
                for (int d = 0; d < D; ++d) wpp[1 + d].add(u[d] * b0);
                if (NDF == 2) wpp[D + 1].add((A)0.5 * wv * (uu * mp[0] + mp[NDF - 1]));
                else wpp[D + 1].add((A)0.5 * uu * b0);
            }
        }
    }
    if (!fst) block_sum_ks<D + 2, NT>(wpp, *reinterpret_cast<double(*)[D + 2]>(wev), sred);
}

// Indices of the per-CTA constants of the flux kernels (shared array sc, arithmetic precision).
enum CellConst {
    C_SDT = 0, C_ADT, C_DS0, C_PREC = C_DS0 + MAXD, C_PREN, C_BFC, C_BFN, C_R1, C_R2, C_SK, C_LC,
    C_UH, C_UL = C_UH + MAXD, C_QA = C_UL + MAXD, C_UNH = C_QA + MAXD, C_UNL = C_UNH + MAXD,
    C_LCH = C_UNL + MAXD, C_LCL, C_LNH, C_LNL, C_N
};

// The scalar section of a cell after its first block reduction: red holds the macro flux
// (red[0 .. D+1]) and the moments of the convected f (red[D+2 ..]).  Two lanes recover the
// conserved update w + dt/V flux with prim_c and the primitives of the convected f (FP64), the
// status bits of prim_c are set, the collision constants go to sc, and the factor tables of the
// two Maxwellians (the second only for CAIDVM marching) are built at Ec.  Ends with the block
// synchronised; sscal holds prim_c (row 0) and the convected f's primitives (row 1).
// we (CIP marching, a donor cell): the moments of the SolidNeighbors' reconstruction
// perturbance, which positivity_preserving_ib! (Boundary/Positivity.jl:1-43) adds to the
// updated w with its limiter factor theta (left in sscal[2 * MAXW]); nullptr otherwise.
// Ec: the factor tables of the two Maxwellians, M_c at Ec[(d * max_axis + a) * TS] and M_n
// after them (TS = 1) or interleaved with them at + 1 (TS = 4, the packed kernel's table)
template <int D, int NDF, typename A, int NT, int TS = 1>
__device__ __forceinline__ void cell_constants(const Dev& P, int cell, int slot, const ProbParams& PP, double dt,
                                               double invV, const double (&red)[2 * (D + 2)], double* sscal, A* sc,
                                               A* Ec, int gid, const double* we = nullptr) {
    const double Kgas = PP.K;
    const int MA = P.max_axis;
    {
        // Two lanes recover the two sets of primitives in one FP64 instruction stream (on
        // GB300 an FP64 warp instruction costs the same for one lane or 32): lane 0 the
        // conserved update w + dt/V·flux and prim_c, lane 1 the primitives of the convected f
        // (Euler: both lanes the same, so prim_n = prim_c)
        if (threadIdx.x < 2) {
            const int ln = threadIdx.x;
            double* w = P.w + (int64_t)cell * MAXW;
            const double dtV = dt * invV;
            const bool lane_mom = P.marching != KG_MARCH_EULER ? ln == 1 : P.flux == KG_FLUX_DVM;
            double wv[MAXW], pv[MAXW];
#pragma unroll
            for (int q = 0; q < D + 2; ++q) wv[q] = lane_mom ? red[D + 2 + q] : fma(red[q], dtV, w[q]);
            if (we && ln == 0) {
                // positivity_preserving_ib!: theta = min(theta_rho, theta_e), margin 1e-3
                double wev[MAXW];
#pragma unroll
                for (int q = 0; q < D + 2; ++q) wev[q] = we[q] * dtV;
                const double delta = 1e-3;
                const double th_rho = wev[0] > 0.0 ? 1.0 : jl_min(1.0, (1.0 - delta) * wv[0] / (fabs(wev[0]) + JL_EPS));
                double rub2 = 0.0, rue2 = 0.0, rbe = 0.0;
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    rub2 += wv[1 + d] * wv[1 + d];
                    rue2 += wev[1 + d] * wev[1 + d];
                    rbe += wv[1 + d] * wev[1 + d];
                }
                const double eb = wv[D + 1] - rub2 / (2.0 * wv[0]);
                const double ee = wev[D + 1] - rbe / wv[0];
                const double gam = rue2 / (2.0 * wv[0]);
                const double th_e = jl_min(1.0, 2.0 * (1.0 - delta) * eb / (sqrt(ee * ee + 4.0 * gam * (1.0 - delta) * eb) - ee + JL_EPS));
                const double th = jl_min(th_rho, th_e);
#pragma unroll
                for (int q = 0; q < D + 2; ++q) wv[q] += th * wev[q];
                sscal[2 * MAXW] = th;
            }
            get_prim_r<D>(wv, PP.gamma, pv);
#pragma unroll
            for (int q = 0; q < D + 2; ++q) sscal[ln * MAXW + q] = pv[q];
            if (ln == 0) {
#pragma unroll
                for (int q = 0; q < D + 2; ++q) w[q] = wv[q];
            }
        }
        if (threadIdx.x < 32) {
            __syncwarp();
            const int lane = threadIdx.x;
            // hi/lo pairs (one lane each, one instruction stream): U_c (lanes 0..D-1),
            // U_n (8..), lambda_c (16), lambda_n (17)
            int src = -1, dh = 0, dl = 0;
            if (lane < D) { src = 1 + lane; dh = C_UH + lane; dl = C_UL + lane; }
            else if (lane >= 8 && lane < 8 + D) { src = MAXW + 1 + lane - 8; dh = C_UNH + lane - 8; dl = C_UNL + lane - 8; }
            else if (lane == 16) { src = D + 1; dh = C_LCH; dl = C_LCL; }
            else if (lane == 17) { src = MAXW + D + 1; dh = C_LNH; dl = C_LNL; }
            if (src >= 0) {
                const double x = sscal[src];
                const A h = (A)x;
                sc[dh] = h;
                sc[dl] = (A)(x - (double)h);
            }
            // status of prim_c: one lane per component
            int bad = 0;
            if (lane < D + 2) {
                const double x = sscal[lane];
                if (!isfinite(x)) bad |= ST_NONFINITE;
                if ((lane == 0 || lane == D + 1) && !(x > 0.0)) bad |= ST_NEGATIVE;
            }
            bad = __reduce_or_sync(0xffffffffu, bad);
            if (lane == 0) {
                if (bad) atomicOr(&P.status[slot], bad);
                const double* pc = sscal;
                const double* pn = sscal + MAXW;
                const double lc = pc[D + 1], ln = pn[D + 1];
                if constexpr (sizeof(A) == 8) {
                    // get_τ (Gas/Model.jl:14) and the constants of discrete_maxwell / shakhov_part
                    const double tau = PP.mu_ref * 2.0 * pow(lc, 1.0 - PP.omega) / pc[0];
                    sc[C_PREC] = pc[0] * (D == 2 ? lc / PI : pow(lc / PI, 1.5));
                    sc[C_PREN] = pn[0] * (D == 2 ? ln / PI : pow(ln / PI, 1.5));
                    sc[C_BFC] = Kgas / (2.0 * lc);
                    sc[C_BFN] = Kgas / (2.0 * ln);
                    sc[C_R1] = tau / (tau + dt);
                    sc[C_R2] = dt / (tau + dt);
                    sc[C_SK] = 0.8 * (1.0 - PP.Pr) * lc * lc / pc[0];
                    sc[C_LC] = lc;
                } else {
                    // mixed form: the same constants in FP32 (they scale FP32 per-velocity values)
                    const float rc = (float)pc[0], rn = (float)pn[0];
                    const float lcf = (float)sc[C_LCH], lnf = (float)sc[C_LNH];
                    const float dtf = PP.dtf;
                    const float tau = PP.mu2f * powf(lcf, PP.omf) / rc;
                    constexpr float IPI = (float)(1.0 / PI);
                    sc[C_PREC] = rc * (D == 2 ? lcf * IPI : powf(lcf * IPI, 1.5f));
                    sc[C_PREN] = rn * (D == 2 ? lnf * IPI : powf(lnf * IPI, 1.5f));
                    sc[C_BFC] = PP.Kf / (2.f * lcf);
                    sc[C_BFN] = PP.Kf / (2.f * lnf);
                    sc[C_R1] = tau / (tau + dtf);
                    sc[C_R2] = dtf / (tau + dtf);
                    sc[C_SK] = PP.shkf * lcf * lcf / rc;
                    sc[C_LC] = lcf;
                }
            }
        }
        __syncthreads();
    }
    // factor tables of the two Maxwellians (discrete_maxwell, 2D2F.jl:1-21 / 3D1F.jl:1-23)
    static_assert(TS == 1 || sizeof(A) == 4, "interleaved tables are FP32");
    const bool need_n = P.marching == KG_MARCH_CAIDVM;
    A* En = TS == 1 ? Ec + (size_t)D * MA : Ec + 1;
    if constexpr (sizeof(A) == 8) {
        gauss_table<D, NT>(P, gid, &sscal[1], sscal[D + 1], (double*)Ec);
        if (need_n) gauss_table<D, NT>(P, gid, &sscal[MAXW + 1], sscal[MAXW + D + 1], (double*)En);
    } else {
        gauss_table<D, NT, TS, TS == 4>(P, gid, (const float*)&sc[C_UH], (const float*)&sc[C_UL], (float)sc[C_LCH], (float)sc[C_LCL], (float*)Ec);
        if (need_n)
            gauss_table<D, NT, TS>(P, gid, (const float*)&sc[C_UNH], (const float*)&sc[C_UNL], (float)sc[C_LNH], (float)sc[C_LNL], (float*)En);
    }
    __syncthreads();
}

// prim_c, the residual terms of residual_check! (Solver/Finalize.jl:5-11) and qf of a cell
// after its collision, one lane per component.
template <int D>
__device__ __forceinline__ void cell_outputs(const Dev& P, int cell, int fcx, int64_t step, int check_interval,
                                             const double* sscal, const double* qv) {
    if (threadIdx.x < MAXW) {
        const int q = threadIdx.x;
        double* pr = P.prim + (int64_t)cell * MAXW;
        double* res = P.cell_res + (int64_t)fcx * 2 * MAXW;
        const bool chk = (step % check_interval) == 0;
        if (q < D + 2) {
            const double pcq = sscal[q];
            const double dl = pcq - pr[q];
            res[q] = chk ? dl * dl : 0.0;
            res[MAXW + q] = chk ? fabs(pcq) : 0.0;
            pr[q] = pcq;
        } else {
            res[q] = 0.0;
            res[MAXW + q] = 0.0;
        }
#pragma unroll
        for (int d = 0; d < D; ++d)
            if (q == d) P.qf[(int64_t)cell * MAXD + d] = 0.5 * qv[d];
    }
}

// the faces of a regular cell (fluid_reg), by direction and side (2*dir + (face at +ds/2))
template <typename A, typename T> struct RegFace {
    const T* of;    // the neighbour's f and sdf blocks
    const T* os;
    A dxm;          // face midpoint - my centre along dir (= -(face midpoint - neighbour's centre))
    A sarea;
};

// flux + collision of fluid cell number fcx (one CTA; every thread of the block takes part).
// FG: the convected f is staged in the cell's output block instead of shared memory (a
// compile-time choice, so that the shared-memory variant keeps shared-memory instructions).
// REG: the cell is regular (fluid_reg): its faces come from its RegRec, with no incidence
// list, and the regular branch of the gather runs.
template <int D, int NDF, typename T, bool FG, int NT, bool REG, bool PPIB = false>
__device__ __forceinline__ void flux_collide_cell(const Dev& P, const int fcx) {
    using A = typename Arith<T>::type;
    extern __shared__ __align__(16) unsigned char sh_raw[];
    __shared__ Incidence sinc[MAX_INC];
    __shared__ IncA<A, T> sia[MAX_INC];
    __shared__ RegFace<A, T> srf[2 * MAXD];
    __shared__ int8_t sbt[MAX_INC];             // incidence -> its Maxwellian factor table, -1 none
    __shared__ A sbpre[MAX_INC], sbk[MAX_INC];  // ρ (λ/π)^{D/2} and K/(2λ) of that Maxwellian
    __shared__ double sred[2 * (D + 2) * (NT / 32)];
    __shared__ double sscal[4 * MAXW];
    // per-CTA scalars in the arithmetic precision (CellConst)
    __shared__ A sc[C_N];
    // one record of the cell, then its incidences: two dependent loads before the barrier
    const FluxCell FC = P.fcrec[fcx];
    if (threadIdx.x == 32) {
        // the cell's own f and sdf blocks into L2 while the block sets up (warp 0 is busy)
        prefetch_l2((const T*)P.f_in + FC.foff, sizeof(T) * (size_t)NDF * FC.nv);
        prefetch_l2((const T*)P.sdf + FC.foff * D, sizeof(T) * (size_t)D * NDF * FC.nv);
    }
    const int cell = FC.cell;
    const int slot = FC.slot;
    const ProbParams& PP = P.probs[slot];
    const double dt = PP.dt;
    const double Kgas = PP.K;
    const int64_t step = P.prob_step[slot];
    const int check_interval = PP.check;
    const int i0 = FC.inc0, ninc = REG ? 0 : FC.ninc;
    // regular cells run the regular-cell kernels only (every schedule routes them there)
    constexpr bool reg = REG;
    for (int e = threadIdx.x; e < ninc; e += NT) {
        const Incidence I = P.inc[i0 + e];
        sinc[e] = I;
        IncA<A, T> ia;
        if constexpr (sizeof(A) == 4) {
#pragma unroll
            for (int d = 0; d < MAXD; ++d) { ia.dxm[d] = I.dxm_f[d]; ia.dxo[d] = I.dxo_f[d]; ia.ods[d] = I.ods_f[d]; }
            ia.orient = I.orient_f;
            ia.sarea = I.sarea_f;
        } else {
#pragma unroll
            for (int d = 0; d < MAXD; ++d) {
                ia.dxm[d] = (A)(I.fmid[d] - I.my_mid[d]);
                ia.dxo[d] = (A)(I.fmid[d] - I.ot_mid[d]);
                ia.ods[d] = (A)I.ot_ds[d];
            }
            ia.orient = (A)I.orient;
            ia.sarea = (A)I.sarea;
        }
        ia.kind = I.kind; ia.dir = I.dir; ia.bc_kind = I.bc_kind; ia.pair = I.pair;
        if (I.kind == INC_DOMAIN) ia.mode_out = (I.bc_kind == KG_BC_OUTFLOW) ? 2 : 1;
        else ia.mode_out = (I.kind == INC_SOLID) ? 1 : 0;
        ia.mode_in = (I.kind == INC_SOLID) ? (P.flux == KG_FLUX_CAIDVM ? 2 : 1) : 0;
        if (I.other >= 0) {
            ia.of = (const T*)P.f_in + I.ofoff;
            ia.os = (const T*)P.sdf + I.ofoff * D;
            ia.onv = I.onv;
            ia.ogo = I.ogo;
        } else {
            ia.of = nullptr; ia.os = nullptr; ia.onv = 0; ia.ogo = 0;
        }
        sia[e] = ia;
        if (reg) {
            // (selects rather than a runtime index keep ia and I in registers)
            const int d = I.dir;
            const A dm = d == 0 ? ia.dxm[0] : (d == 1 ? ia.dxm[1] : ia.dxm[MAXD - 1]);
            RegFace<A, T> rf;
            rf.of = ia.of; rf.os = ia.os; rf.dxm = dm; rf.sarea = ia.sarea;
            srf[2 * d + (dm > (A)0 ? 1 : 0)] = rf;
        }
    }
    if constexpr (REG) {
        // the faces of a regular cell from its RegRec, by side 2 * dir + (face at +ds/2)
        if (threadIdx.x < 2 * D) {
            const int q = threadIdx.x;
            const RegRec& RR = P.regrec[fcx];
            RegFace<A, T> rf;
            rf.of = (const T*)P.f_in + RR.nfo[q];
            rf.os = (const T*)P.sdf + RR.nfo[q] * D;
            if constexpr (sizeof(A) == 4) { rf.dxm = RR.dxm_f[q]; rf.sarea = RR.sa_f[q]; }
            else { rf.dxm = (A)RR.dxm[q]; rf.sarea = (A)RR.sa[q]; }
            srf[q] = rf;
        }
    }
    const double invV = FC.invV;
    if (threadIdx.x == 0) {
        sc[C_SDT] = (A)(dt * invV);
        sc[C_ADT] = (A)dt;
        for (int d = 0; d < D; ++d) sc[C_DS0 + d] = (A)FC.ds[d];
    }
    __syncthreads();
    VGridView g;
    g.goff = FC.goff;
    g.nv = FC.nv;
    g.vu = P.vu;
    g.PG = P.PG;
    const int nv = g.nv;
    const int gid = FC.gid;
    const int64_t PG = P.PG;
    const A* VU = vel<A>(P);
    const A* VW0 = wts<A>(P);
    const A* VW = VW0 + g.goff;
    const int64_t fo = FC.foff;
    const T* fcell = (const T*)P.f_in + fo;
    const T* scl = (const T*)P.sdf + fo * D;
    T* fnew = (T*)P.f_out + fo;
    A myds[D];
#pragma unroll
    for (int d = 0; d < D; ++d) myds[d] = sc[C_DS0 + d];
    const A s_dt = sc[C_SDT];
    const A adt = sc[C_ADT];
    // convected f, NDF * nv: in shared memory, or -- when that would cost resident CTAs (large
    // 3D grids) -- in the cell's output block, which stays in L2 until the relaxation
    // overwrites it; every access below is by the thread that owns velocity i, at k * nv + i
    static_assert(sizeof(A) == sizeof(T), "the staging block holds the arithmetic type");
    A* fst = FG ? (A*)fnew : (A*)sh_raw;
    A* Ec = FG ? (A*)sh_raw : fst + (size_t)NDF * nv;   // factor tables (flux_smem)
    const bool caidvm = P.flux == KG_FLUX_CAIDVM;

    const int MA = P.max_axis;
    const uint16_t* vx = P.vidx + g.goff;

    // ---- 0. Maxwellians of the domain faces with a Maxwellian state (wall, inflow) ---------
    // Per such face: factor tables of exp(-λ|u-U|²) at the grid's axis coordinates (in the
    // region of the collision tables, which are built after the flux), the prefactor
    // ρ (λ/π)^{D/2} and K/(2λ).  A wall face's density is calc_ρw (Theory/Math.jl:251-282):
    // ρ_w = -Σ_out w u_n f̂ / ((λ/π)^{D/2} Σ_in w u_n e^{-λ|u-U|²}).
    int nbt = 0;
    for (int e = 0; e < ninc; ++e) {
        const Incidence& I = sinc[e];
        const bool tab = I.kind == INC_DOMAIN && (I.bc_kind == KG_BC_MAXWELL || I.bc_kind == KG_BC_INFLOW);
        if (threadIdx.x == 0) sbt[e] = tab ? (int8_t)nbt : (int8_t)-1;
        if (!tab) continue;
        A* Eb = Ec + (size_t)nbt * D * MA;
        if constexpr (sizeof(A) == 8) {
            const double* bc = P.bc_prim + (int64_t)I.bc * MAXW;
            gauss_table<D, NT>(P, gid, bc + 1, bc[D + 1], (double*)Eb);
        } else {
            const float* hl = P.bc_hl + (int64_t)I.bc * 2 * MAXW;
            gauss_table<D, NT>(P, gid, hl + 1, hl + MAXW + 1, hl[D + 1], hl[MAXW + D + 1], (float*)Eb);
        }
        ++nbt;
    }
    if (nbt > 0) {
        __syncthreads();
        for (int e = 0; e < ninc; ++e) {
            const Incidence& I = sinc[e];
            const int b = sbt[e];
            if (b < 0) continue;
            const double* bc = P.bc_prim + (int64_t)I.bc * MAXW;
            if (I.bc_kind == KG_BC_MAXWELL) {
                const A* Eb = Ec + (size_t)b * D * MA;
                KSum<A> red[2];
                for (int i = threadIdx.x; i < nv; i += NT) {
                    const A ud = VU[(int64_t)I.dir * PG + g.goff + i];
                    if (sia[e].orient * ud <= (A)0) {
                        const A fk = (A)fcell[i];
                        A sl[D], dx[D];
#pragma unroll
                        for (int d = 0; d < D; ++d) {
                            sl[d] = (A)scl[(int64_t)d * NDF * nv + i];
                            dx[d] = sia[e].dxm[d] - VU[(int64_t)d * PG + g.goff + i] * adt;
                        }
                        red[0].add(VW[i] * ud * own_recon<D, A>(1, fk, sl, dx, myds));
                    } else {
                        A shape = (A)1;
#pragma unroll
                        for (int d = 0; d < D; ++d) shape *= Eb[d * MA + vx[(int64_t)d * PG + i]];
                        red[1].add(VW[i] * ud * shape);
                    }
                }
                double rs[2];
                block_sum_ks<2, NT>(red, rs, sred);
                if (threadIdx.x == 0) {
                    const double lam = bc[D + 1];
                    const double pre = D == 2 ? lam / PI : pow(lam / PI, 1.5);
                    const double rho = -rs[0] / (pre * rs[1]);
                    sbpre[e] = (A)(rho * pre);
                    sbk[e] = (A)(Kgas / (2.0 * lam));
                }
            } else if (threadIdx.x == 0) {
                const double lam = bc[D + 1];
                sbpre[e] = (A)(bc[0] * (D == 2 ? lam / PI : pow(lam / PI, 1.5)));
                sbk[e] = (A)(Kgas / (2.0 * lam));
            }
        }
        __syncthreads();
    }

    // ---- 1. fluxes gathered over the incidences; convected f into shared memory ----
    KSum<A> wacc[D + 2], wfc[D + 2];
    // CIP marching, a donor cell: positivity_preserving_ib! (one uniform flag per CTA)
    // (PPIB: the kernel variant of CIP-marching layouts with walls, so that no other layout
    // carries this code)
    bool pp_ib = false;
    if constexpr (PPIB)
        for (int e = 0; e < ninc; ++e) pp_ib |= sinc[e].wallrec != 0;
    for (int i = threadIdx.x; i < nv; i += NT) {
        A u[D];
#pragma unroll
        for (int d = 0; d < D; ++d) u[d] = VU[(int64_t)d * PG + g.goff + i];
        A fr[NDF], sr[NDF][D];
#pragma unroll
        for (int k = 0; k < NDF; ++k) {
            fr[k] = (A)fcell[k * nv + i];
#pragma unroll
            for (int d = 0; d < D; ++d) sr[k][d] = (A)scl[(d * NDF + k) * nv + i];
        }
        A acc[NDF], accM[NDF];
#pragma unroll
        for (int k = 0; k < NDF; ++k) { acc[k] = 0; accM[k] = 0; }
        if (reg) {
            // regular cell: per direction the velocity leaves through the face it points at
            // (own reconstruction there) and enters through the opposite face (the upwind
            // neighbour's reconstruction) -- the generic loop below with its branches resolved;
            // the own limiter factor (positivity_preserving_reconstruct, the same for every
            // face) once per velocity
            A thown[NDF];
#pragma unroll
            for (int k = 0; k < NDF; ++k) {
                A sabs = 0;
#pragma unroll
                for (int d = 0; d < D; ++d) sabs += myds[d] * fabs(sr[k][d]);
                const A th = fabs(lim_div(fr[k] - (A)JL_EPS, (A)0.5 * sabs + (A)EPS_REF));
                thown[k] = th < (A)1 ? th : (A)1;
            }
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const A ud = u[d];
                const int so = 2 * d + (ud > (A)0 ? 1 : 0);
                const RegFace<A, T>& fo_ = srf[so];
                const RegFace<A, T>& fi_ = srf[so ^ 1];
                A dx[D], dxo[D];
#pragma unroll
                for (int d2 = 0; d2 < D; ++d2) {
                    dx[d2] = (d2 == d ? fo_.dxm : (A)0) - u[d2] * adt;
                    dxo[d2] = d2 == d ? -fi_.dxm : (A)0;
                }
                A mi[NDF];
                other_micro<D, NDF, T, A>(fi_.of, fi_.os, nv, i, u, dxo, myds, adt, d, 0, mi);
#pragma unroll
                for (int k = 0; k < NDF; ++k) {
                    A sdx = 0;
#pragma unroll
                    for (int d2 = 0; d2 < D; ++d2) sdx += dx[d2] * sr[k][d2];
                    const A mo = (fr[k] + thown[k] * sdx) * ud;
                    acc[k] += fo_.sarea * mo;
                    acc[k] += fi_.sarea * mi[k];
                }
            }
#pragma unroll
            for (int k = 0; k < NDF; ++k) accM[k] = acc[k];
        } else
        for (int e = 0; e < ninc; ++e) {
            const IncA<A, T>& ia = sia[e];
            const int dir = ia.dir;
            const A ud = D == 2 ? (dir == 0 ? u[0] : u[D - 1]) : (dir == 0 ? u[0] : (dir == 1 ? u[1] : u[D - 1]));
            const A sa = ia.sarea;
            if (ia.orient * ud <= (A)0) {
                // outgoing from this cell: its own reconstruction at the face
                A dx[D];
#pragma unroll
                for (int d = 0; d < D; ++d) dx[d] = ia.dxm[d] - u[d] * adt;
                const int mode = ia.mode_out;
#pragma unroll
                for (int k = 0; k < NDF; ++k) {
                    const A m = own_recon<D, A>(mode, fr[k], sr[k], dx, myds) * ud;
                    acc[k] += sa * m;
                    accM[k] += sa * m;
                }
            } else if (ia.kind != INC_DOMAIN && ia.pair < 0) {
                // incoming through a face to a cell on the same grid (the common case)
                A m[NDF];
                other_micro<D, NDF, T, A>(ia.of, ia.os, ia.onv, i, u, ia.dxo, ia.ods, adt, dir, ia.mode_in, m);
#pragma unroll
                for (int k = 0; k < NDF; ++k) { acc[k] += sa * m[k]; accM[k] += sa * m[k]; }
            } else if (ia.kind == INC_DOMAIN) {
                const Incidence& I = sinc[e];
                A mic[NDF];
                if (I.bc_kind == KG_BC_MAXWELL || I.bc_kind == KG_BC_INFLOW) {
                    const A* Eb = Ec + (size_t)sbt[e] * D * MA;
                    A mh = sbpre[e];
#pragma unroll
                    for (int d = 0; d < D; ++d) mh *= Eb[d * MA + vx[(int64_t)d * PG + i]];
                    mic[0] = mh * ud;
                    if (NDF == 2) mic[NDF - 1] = mh * sbk[e] * ud;
                } else if (I.bc_kind == KG_BC_OUTFLOW) {
#pragma unroll
                    for (int k = 0; k < NDF; ++k) mic[k] = fr[k] * ud;
                } else {  // interpolated outflow (CAIDVM.jl:71-94): mirror centre 2*face - centre
                    A tdx[D];
#pragma unroll
                    for (int d = 0; d < D; ++d) tdx[d] = -ia.dxm[d] - u[d] * adt;
                    const A shift = (A)2 * ia.dxm[dir];
#pragma unroll
                    for (int k = 0; k < NDF; ++k) {
                        const A sdir = D == 2 ? (dir == 0 ? sr[k][0] : sr[k][D - 1])
                                              : (dir == 0 ? sr[k][0] : (dir == 1 ? sr[k][1] : sr[k][D - 1]));
                        A tdf = fr[k] + shift * sdir;
                        mic[k] = own_recon<D, A>(1, tdf, sr[k], tdx, myds) * ud;
                    }
                }
#pragma unroll
                for (int k = 0; k < NDF; ++k) { acc[k] += sa * mic[k]; accM[k] += sa * mic[k]; }
            } else {
                // incoming from a cell on a different velocity grid: mapped through the pairing
                const int li = P.vlev[g.goff + i];
                const int64_t po = P.p_off[ia.pair] + i;
                const int j0 = P.p_j0[po], jc = P.p_cnt[po];
                A mic[NDF];
#pragma unroll
                for (int k = 0; k < NDF; ++k) mic[k] = 0;
                for (int j = j0; j < j0 + jc; ++j) {
                    A uj[D], m[NDF];
#pragma unroll
                    for (int d = 0; d < D; ++d) uj[d] = VU[(int64_t)d * PG + ia.ogo + j];
                    other_micro<D, NDF, T, A>(ia.of, ia.os, ia.onv, j, uj, ia.dxo, ia.ods, adt, dir, ia.mode_in, m);
                    const A sc = merge_scale<D, A>(li, P.vlev[ia.ogo + j]);
#pragma unroll
                    for (int k = 0; k < NDF; ++k) mic[k] += m[k] * sc;
                }
#pragma unroll
                for (int k = 0; k < NDF; ++k) acc[k] += sa * mic[k];
            }
        }
        const A wi = VW[i];
        A fs[NDF];
#pragma unroll
        for (int k = 0; k < NDF; ++k) {
            fs[k] = fr[k] + s_dt * acc[k];
            fst[(int64_t)k * nv + i] = fs[k];
        }
        // macro flux of this grid's micro fluxes: Σ_faces area w ψ micro = w ψ Σ_faces area micro
        A u2 = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) u2 += u[d] * u[d];
        if (caidvm) {
            const A a0 = wi * accM[0];
            wacc[0].add(a0);
#pragma unroll
            for (int d = 0; d < D; ++d) wacc[1 + d].add(u[d] * a0);
            if (NDF == 2) wacc[D + 1].add((A)0.5 * wi * (u2 * accM[0] + accM[NDF - 1]));
            else wacc[D + 1].add((A)0.5 * u2 * a0);
        }
        // CAIDVM: moments of the convected f; Euler: moments of f before convection
        const A* mf = (P.marching == KG_MARCH_CAIDVM) ? fs : fr;
        const A b0 = wi * mf[0];
        wfc[0].add(b0);
#pragma unroll
        for (int d = 0; d < D; ++d) wfc[1 + d].add(u[d] * b0);
        if (NDF == 2) wfc[D + 1].add((A)0.5 * wi * (u2 * mf[0] + mf[NDF - 1]));
        else wfc[D + 1].add((A)0.5 * u2 * b0);
    }
    // macro flux of incoming halves on a different grid (moments on the other side's grid)
    if (caidvm) {
        for (int e = 0; e < ninc; ++e) {
            const Incidence& I = sinc[e];
            if (I.kind == INC_DOMAIN || I.pair < 0) continue;
            const int od = I.other;
            const VGridView go = grid_view(P, od);
            const int onv = go.nv;
            const T* of = sia[e].of;
            const T* os = sia[e].os;
            const int mode = sia[e].mode_in;
            for (int j = threadIdx.x; j < onv; j += NT) {
                A uj[D];
#pragma unroll
                for (int d = 0; d < D; ++d) uj[d] = VU[(int64_t)d * PG + go.goff + j];
                if (sia[e].orient * uj[I.dir] <= (A)0) continue;   // not leaving the other side towards us
                A m[NDF];
                other_micro<D, NDF, T, A>(of, os, onv, j, uj, sia[e].dxo, sia[e].ods, adt, I.dir, mode, m);
                const A wj = VW0[go.goff + j] * sia[e].sarea;
                A u2 = 0;
#pragma unroll
                for (int d = 0; d < D; ++d) u2 += uj[d] * uj[d];
                const A a0 = wj * m[0];
                wacc[0].add(a0);
#pragma unroll
                for (int d = 0; d < D; ++d) wacc[1 + d].add(uj[d] * a0);
                if (NDF == 2) wacc[D + 1].add((A)0.5 * wj * (u2 * m[0] + m[NDF - 1]));
                else wacc[D + 1].add((A)0.5 * u2 * a0);
            }
        }
    }
    // ---- 2. cell scalars ---------------------------------------------------------
    {
        double red[2 * (D + 2)];
        {
            KSum<A> both[2 * (D + 2)];
#pragma unroll
            for (int q = 0; q < D + 2; ++q) { both[q] = wacc[q]; both[D + 2 + q] = wfc[q]; }
            block_sum_ks<2 * (D + 2), NT>(both, red, sred);
        }
        double wev[D + 2];
        if constexpr (PPIB)
            if (pp_ib) pp_ib_pass<D, NDF, T, NT>(sinc, sia, ninc, nv, VU + g.goff, PG, VW, adt, (A)0, nullptr, wev, sred);
        cell_constants<D, NDF, A, NT>(P, cell, slot, PP, dt, invV, red, sscal, sc, Ec, gid, (PPIB && pp_ib) ? wev : nullptr);
    }
    // the limited perturbance joins the convected f: f += dt/V theta micro (the velocity-space
    // flux of iterate!(CIP_Marching), I-projection.jl:176)
    if constexpr (PPIB)
        if (pp_ib) pp_ib_pass<D, NDF, T, NT>(sinc, sia, ninc, nv, VU + g.goff, PG, VW, adt, s_dt * (A)sscal[2 * MAXW], fst, nullptr, sred);
    const bool need_n = P.marching == KG_MARCH_CAIDVM;
    A* En = Ec + (size_t)D * MA;
    const A prec = sc[C_PREC], pren = sc[C_PREN];
    const A bfc = sc[C_BFC], bfn = sc[C_BFN];
    // peculiar velocity c = u - U with U split into two floats (hi + lo), so that c keeps
    // the precision of c rather than that of U
    A Uh[D], Ul[D];
#pragma unroll
    for (int d = 0; d < D; ++d) { Uh[d] = sc[C_UH + d]; Ul[d] = sc[C_UL + d]; }
    // ---- 3. conservation correction and heat flux --------------------------------
    KSum<A> qs[D];
    // heat_flux_2D2F / 3D1F (lib/KitCore/2D2F.jl:68-88, 3D1F.jl:41-72) of f at velocity i
    auto qadd = [&](int i, const A* fv) {
        A c[D], c2 = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) { c[d] = (VU[(int64_t)d * PG + g.goff + i] - Uh[d]) - Ul[d]; c2 += c[d] * c[d]; }
        const A wi = VW[i];
        const A hb = NDF == 2 ? (c2 * fv[0] + fv[NDF - 1]) : c2 * fv[0];
#pragma unroll
        for (int d = 0; d < D; ++d) qs[d].add(wi * c[d] * hb);
    };
    if (need_n) {
        // conservation correction f += M(prim_c) - M(prim)  (Theory/Iterate.jl:117), then q
        for (int i = threadIdx.x; i < nv; i += NT) {
            A mc = prec, mn = pren;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const int ix = vx[(int64_t)d * PG + i];
                mc *= Ec[d * MA + ix];
                mn *= En[d * MA + ix];
            }
            A fv[NDF];
            fv[0] = fst[i] + (mc - mn);
            if (NDF == 2) fv[NDF - 1] = fst[nv + i] + (mc * bfc - mn * bfn);
#pragma unroll
            for (int k = 0; k < NDF; ++k) fst[k * nv + i] = fv[k];
            qadd(i, fv);
        }
    } else if (P.marching == KG_MARCH_CIP) {
        // CIP: q of the convected f (Theory/I-projection.jl:178)
        for (int i = threadIdx.x; i < nv; i += NT) {
            A fv[NDF];
#pragma unroll
            for (int k = 0; k < NDF; ++k) fv[k] = fst[k * nv + i];
            qadd(i, fv);
        }
    } else {
        // Euler: q of f before convection (Theory/Iterate.jl:153)
        for (int i = threadIdx.x; i < nv; i += NT) {
            A fv[NDF];
#pragma unroll
            for (int k = 0; k < NDF; ++k) fv[k] = (A)fcell[k * nv + i];
            qadd(i, fv);
        }
    }
    double qv[D];
    block_sum_ks<D, NT>(qs, qv, sred);
    if (threadIdx.x == 0)
        for (int d = 0; d < D; ++d) sc[C_QA + d] = (A)(0.5 * qv[d]);
    __syncthreads();
    // ---- 4. Shakhov g+ and implicit relaxation -------------------------------------
    const A r1 = sc[C_R1], r2 = sc[C_R2];
    const A sk = sc[C_SK];
    const A lc = sc[C_LC], Kk = (A)Kgas;
    A qa[D];
#pragma unroll
    for (int d = 0; d < D; ++d) qa[d] = sc[C_QA + d];
    // g+ = M_c (1 + Shakhov(q)) at velocity i (shakhov_part_2D2F / 3D1F)
    auto gplus = [&](int i, A* gp) {
        A mc = prec;
#pragma unroll
        for (int d = 0; d < D; ++d) mc *= Ec[d * MA + vx[(int64_t)d * PG + i]];
        A c2 = 0, cq = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const A cd = (VU[(int64_t)d * PG + g.goff + i] - Uh[d]) - Ul[d];
            c2 += cd * cd;
            cq += cd * qa[d];
        }
        if (NDF == 2) {
            const A mb = mc * bfc;
            gp[0] = mc + sk * cq * ((A)2 * lc * c2 + Kk - (A)5) * mc;
            gp[NDF - 1] = mb + sk * cq * ((A)2 * lc * c2 + Kk - (A)3) * mb;
        } else {
            gp[0] = mc + sk * cq * ((A)2 * lc * c2 - (A)5) * mc;
        }
    };
    if (P.marching == KG_MARCH_CIP) {
        // the I-projection and the relaxation follow in cip_kernel, from the convected f
        if (!FG)
            for (int i = threadIdx.x; i < nv; i += NT)
#pragma unroll
                for (int k = 0; k < NDF; ++k) fnew[k * nv + i] = (T)fst[k * nv + i];
    } else if (P.marching == KG_MARCH_CAIDVM) {
        // f = f tau/(tau+dt) + dt/(tau+dt) g+   (Theory/Iterate.jl:121-122)
        for (int i = threadIdx.x; i < nv; i += NT) {
            A gp[NDF];
            gplus(i, gp);
#pragma unroll
            for (int k = 0; k < NDF; ++k) fnew[k * nv + i] = (T)(fst[k * nv + i] * r1 + r2 * gp[k]);
        }
    } else {
        // f = (f + dt/V flux) tau/(tau+dt) + dt/(tau+dt) g+   (Theory/Iterate.jl:156)
        for (int i = threadIdx.x; i < nv; i += NT) {
            A gp[NDF];
            gplus(i, gp);
#pragma unroll
            for (int k = 0; k < NDF; ++k) fnew[k * nv + i] = (T)(fst[k * nv + i] * r1 + r2 * gp[k]);
        }
    }
    // ---- 5. per-cell outputs and residual terms ------------------------------------
    cell_outputs<D>(P, cell, fcx, step, check_interval, sscal, qv);
}

// ---- packed-FP32 regular-cell kernel (2D, two distributions, mixed form) ---------------
#ifndef KG_PACKED_VPT
#define KG_PACKED_VPT 2
#endif
#ifndef KG_PACKED_MINB
#define KG_PACKED_MINB 3
#endif
constexpr int PACKED_VPT = KG_PACKED_VPT;   // velocity cells per thread and gather pass
constexpr int R2_VPT = 1;       // the same for the kernel that computes the slopes (more loads a cell)
// Blackwell's FP32x2 instructions (__ffma2_rn / __fmul2_rn / __fadd2_rn: two FP32 lanes per
// thread instruction, each rounded as the scalar instruction) carry the pair (h, b) of every
// velocity cell through the reconstruction, the fluxes, the correction and the relaxation, and
// the pair (macro flux, moments of the convected f) through the moment sums, so a velocity
// cell issues about half the FP32 instructions of the scalar form.  The per-thread moment
// sums are plain FP32 (a thread adds at most a few tens of terms; the block reduction that
// follows is float-float).
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 abs2(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }

// positivity_preserving_reconstruct (Flux/CAIDVM.jl:127-142) of the pair f with slopes s0, s1
// (directions 0 and 1) and cell sizes ds0, ds1: the limiter factor per lane
__device__ __forceinline__ float2 pp_theta2(float2 f, float2 s0, float2 s1, float ds0, float ds1) {
    const float2 sabs = fma2(bc2(ds1), abs2(s1), mul2(bc2(ds0), abs2(s0)));
    const float2 den = fma2(bc2(0.5f), sabs, bc2((float)EPS_REF));
    const float2 num = add2(f, bc2(-(float)JL_EPS));
    return make_float2(fminf(fabsf(__fdividef(num.x, den.x)), 1.f), fminf(fabsf(__fdividef(num.y, den.y)), 1.f));
}

// minmod of each lane, and the regular slope (f - f_n) inv of a pair (slope_kernel's arithmetic:
// the same bits)
__device__ __forceinline__ float2 minmod2(float2 a, float2 b) { return make_float2(minmod(a.x, b.x), minmod(a.y, b.y)); }
__device__ __forceinline__ float2 dslope2(float2 f, float2 fn, float inv) { return mul2(fma2(fn, bc2(-1.f), f), bc2(inv)); }

// R2: the cell's slopes and its upwind neighbours' are computed here from f (R2Rec), so no sdf is read.
// INNER: a cell whose faces are all inner faces to fluid cells, one or two sub-faces a side
// (hanging faces, neighbours of other sizes or on other velocity grids: packed_inner_ok); per
// velocity and direction the sub-faces of the side it leaves through take its own
// reconstruction, those of the side it enters through the neighbour's (INNER = 2: through the
// pairing runs from another grid, whose macro flux is then summed on that grid; INNER = 1: every
// neighbour on the cell's own grid).
struct PSub {                 // one sub-face of a side (INNER): the incidence's FP32 geometry
    float dxm0, dxm1, dxo0, dxo1, ods0, ods1, sa;
    int32_t pair;             // pairing (my grid <- the neighbour's), -1: the same grid
    int64_t poff;             // that pairing's rows (p_off), read once per cell
    int64_t ofoff;            // the neighbour's f offset
    int32_t onv, ogo;         // its velocity count and grid offset
};
template <int NT, int VPT, bool R2, int INNER = 0>
__device__ __forceinline__ void flux_regular_packed(const Dev& P, const int fcx) {
    constexpr int D = 2;
    extern __shared__ __align__(16) unsigned char sh_raw[];
    __shared__ double sred[2 * (D + 2) * (NT / 32)];
    __shared__ double sscal[4 * MAXW];
    __shared__ float sc[C_N];
    __shared__ int64_t nfo[4];
    __shared__ PSub psub[INNER ? 4 : 1][INNER ? 2 : 1];
    __shared__ int pcnt[INNER ? 4 : 1];
    const FluxCell FC = P.fcrec[fcx];
    const int nv = FC.nv;
    if (threadIdx.x == 32) {
        prefetch_l2((const float*)P.f_in + FC.foff, sizeof(float) * (size_t)2 * nv);
        prefetch_l2((const float*)P.sdf + FC.foff * D, sizeof(float) * (size_t)D * 2 * nv);
    }
    const int cell = FC.cell, slot = FC.slot;
    const ProbParams& PP = P.probs[slot];
    const double dt = PP.dt;
    const int64_t step = P.prob_step[slot];
    if (threadIdx.x == 0) {
        sc[C_SDT] = (float)(dt * FC.invV);
        sc[C_ADT] = (float)dt;
        sc[C_DS0] = (float)FC.ds[0];
        sc[C_DS0 + 1] = (float)FC.ds[1];
    }
    // the four faces (side 2 * dir + (face at +ds/2)): neighbour f offset (shared memory),
    // dxm and area factor (registers)
    const RegRec& RR = P.regrec[fcx];
    if (!INNER && threadIdx.x < 4) nfo[threadIdx.x] = RR.nfo[threadIdx.x];
    if constexpr (INNER) {
        // the sub-faces by side (the incidences of such a cell: at most 2 a side, checked)
        if (threadIdx.x == 0) {
            int cnt[4] = {0, 0, 0, 0};
            for (int e = 0; e < FC.ninc; ++e) {
                const Incidence& a = P.inc[FC.inc0 + e];
                const int d = a.dir;
                const int sd = 2 * d + (a.dxm_f[d] > 0.f ? 1 : 0);
                const int k = cnt[sd] < 2 ? cnt[sd]++ : 1;
                PSub q;
                q.dxm0 = a.dxm_f[0]; q.dxm1 = a.dxm_f[1]; q.dxo0 = a.dxo_f[0]; q.dxo1 = a.dxo_f[1];
                q.ods0 = a.ods_f[0]; q.ods1 = a.ods_f[1]; q.sa = a.sarea_f; q.pair = a.pair; q.ofoff = a.ofoff;
                q.poff = a.pair >= 0 ? P.p_off[a.pair] : 0;
                q.onv = a.onv; q.ogo = a.ogo;
                psub[sd][k] = q;
            }
            for (int sd = 0; sd < 4; ++sd) pcnt[sd] = cnt[sd];
        }
    }
    // R2: the neighbours' neighbours and slope factors, and the cell's own slope factors
    __shared__ int64_t snn[R2 ? 16 : 1];
    __shared__ float sninv[R2 ? 16 : 1], ssinv[R2 ? 4 : 1];
    if constexpr (R2) {
        const R2Rec& Q = P.r2rec[fcx];
        if (threadIdx.x < 16) {
            snn[threadIdx.x] = Q.nn[threadIdx.x / 4][threadIdx.x % 4];
            sninv[threadIdx.x] = Q.ninv[threadIdx.x / 4][threadIdx.x % 4];
        }
        if (threadIdx.x < 4) ssinv[threadIdx.x] = Q.sinv[threadIdx.x];
    }
    float rdm[4], rsa[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) { rdm[q] = INNER ? 0.f : RR.dxm_f[q]; rsa[q] = INNER ? 0.f : RR.sa_f[q]; }
    // per axis entry a of the grid: (M_c factor, M_n factor, u_d, c_d) in one 16-byte record, so
    // a velocity's metadata is its two axis indices and its weight (8 bytes) and one shared
    // load per axis (the u_d here are the FP32 velocities of the grid, bit for bit)
    float2* fst = reinterpret_cast<float2*>(sh_raw);               // convected (h, b) per velocity
    float4* T4 = reinterpret_cast<float4*>(sh_raw + packed_table_off(nv));
    const int MA = P.max_axis;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const int a0 = P.ax_off[FC.gid * MAXD + d], na = P.ax_off[FC.gid * MAXD + d + 1] - a0;
        for (int a = threadIdx.x; a < na; a += NT) T4[d * MA + a].z = P.ax_hi[a0 + a];
    }
    __syncthreads();
    const float s_dt = sc[C_SDT], adt = sc[C_ADT], ds0 = sc[C_DS0], ds1 = sc[C_DS0 + 1];
    const float* fbase = (const float*)P.f_in;
    const float* sbase = (const float*)P.sdf;
    const float* fc = fbase + FC.foff;
    const float* scl = sbase + FC.foff * D;
    const uint16_t* vxa = P.vidx + FC.goff;           // axis indices of the velocities
    const uint16_t* vxb = P.vidx + P.PG + FC.goff;
    const float* vwt = P.vwf + FC.goff;               // weights
    // (u_x, u_y, weight, -) of velocity i
    auto vel = [&](int i) {
        const int ix = vxa[i], iy = vxb[i];
        return make_float4(T4[ix].z, T4[MA + iy].z, vwt[i], 0.f);
    };
    const bool caidvm = P.flux == KG_FLUX_CAIDVM;
    const bool march_caidvm = P.marching == KG_MARCH_CAIDVM;

    // ---- 1. the fluxes through the four faces and the convected f ----------------------
    // accumulators of the pairs (macro flux, moments of the convected f): ρ, ρU_x, ρU_y, ρE
    float2 m0 = bc2(0.f), m1 = bc2(0.f), m2 = bc2(0.f), mE = bc2(0.f);
    // the flux sum acc and f of velocity i (loads first, so that VPT velocities' loads are in
    // flight together)
    auto gather = [&](int i, const float4& V, float2& f2, float2& acc) {
        const float u0 = V.x, u1 = V.y;
        f2 = make_float2(fc[i], fc[nv + i]);
        float2 s0, s1, g2[D], t0[D], t1[D];
        if constexpr (R2) {
            // f of the four neighbours and, per direction, of the upwind neighbour's other
            // neighbours (along the direction the far one, across it both); the slopes follow
            float2 fn[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float* o = fbase + nfo[q];
                fn[q] = make_float2(o[i], o[nv + i]);
            }
            float2 ffar[D], fxa[D], fxb[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const bool pos = (d == 0 ? u0 : u1) > 0.f;
                const int su = 2 * d + (pos ? 0 : 1);
                const int e = 1 - d;   // the direction across
                const float* oa = fbase + snn[4 * su + su];
                const float* ob = fbase + snn[4 * su + 2 * e];
                const float* oc = fbase + snn[4 * su + 2 * e + 1];
                ffar[d] = make_float2(oa[i], oa[nv + i]);
                fxa[d] = make_float2(ob[i], ob[nv + i]);
                fxb[d] = make_float2(oc[i], oc[nv + i]);
            }
            s0 = minmod2(dslope2(f2, fn[0], ssinv[0]), dslope2(f2, fn[1], ssinv[1]));
            s1 = minmod2(dslope2(f2, fn[2], ssinv[2]), dslope2(f2, fn[3], ssinv[3]));
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const bool pos = (d == 0 ? u0 : u1) > 0.f;
                const int su = 2 * d + (pos ? 0 : 1);
                const int e = 1 - d;
                const float2 gn = fn[su];
                g2[d] = gn;
                // along d: the neighbour's far side is side su, the cell itself the other
                const float2 fa = (su & 1) ? f2 : ffar[d];
                const float2 fb = (su & 1) ? ffar[d] : f2;
                const float2 sd = minmod2(dslope2(gn, fa, sninv[4 * su + 2 * d]), dslope2(gn, fb, sninv[4 * su + 2 * d + 1]));
                const float2 se = minmod2(dslope2(gn, fxa[d], sninv[4 * su + 2 * e]), dslope2(gn, fxb[d], sninv[4 * su + 2 * e + 1]));
                t0[d] = d == 0 ? sd : se;
                t1[d] = d == 0 ? se : sd;
            }
        } else {
            s0 = make_float2(scl[i], scl[nv + i]);
            s1 = make_float2(scl[2 * nv + i], scl[3 * nv + i]);
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const bool pos = (d == 0 ? u0 : u1) > 0.f;
                const int64_t no = nfo[2 * d + (pos ? 0 : 1)];
                const float* of = fbase + no;
                const float* os = sbase + no * D;
                g2[d] = make_float2(of[i], of[nv + i]);
                t0[d] = make_float2(os[i], os[nv + i]);
                t1[d] = make_float2(os[2 * nv + i], os[3 * nv + i]);
            }
        }
        const float2 th = pp_theta2(f2, s0, s1, ds0, ds1);
        acc = bc2(0.f);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const float ud = d == 0 ? u0 : u1;
            const bool pos = ud > 0.f;
            // outgoing through the face the velocity points at: the own reconstruction
            const float dmo = pos ? rdm[2 * d + 1] : rdm[2 * d];
            const float sao = pos ? rsa[2 * d + 1] : rsa[2 * d];
            const float dx0 = (d == 0 ? dmo : 0.f) - u0 * adt;
            const float dx1 = (d == 1 ? dmo : 0.f) - u1 * adt;
            const float2 sdx = fma2(bc2(dx1), s1, mul2(bc2(dx0), s0));
            const float2 mo = mul2(fma2(th, sdx, f2), bc2(ud));
            acc = fma2(bc2(sao), mo, acc);
            // incoming through the opposite face: the upwind neighbour's reconstruction
            const float dmi = pos ? rdm[2 * d] : rdm[2 * d + 1];
            const float sai = pos ? rsa[2 * d] : rsa[2 * d + 1];
            const float ndx0 = (d == 0 ? -dmi : 0.f) - u0 * adt;
            const float ndx1 = (d == 1 ? -dmi : 0.f) - u1 * adt;
            const float2 nsdx = fma2(bc2(ndx1), t1[d], mul2(bc2(ndx0), t0[d]));
            const float2 thn = pp_theta2(g2[d], t0[d], t1[d], ds0, ds1);
            const float2 mi = mul2(fma2(thn, nsdx, g2[d]), bc2(ud));
            acc = fma2(bc2(sai), mi, acc);
        }
    };
    // INNER: the flux sum of velocity i through the sub-faces of the four sides (the loads of
    // the two sides it enters through first)
    // the micro flux into this cell at velocity i through paired sub-face q: the neighbour's
    // reconstructed micro fluxes at the velocities of its grid that overlap i (the pairing run),
    // averaged onto i (a finer run) or copied (a coarser or equal one)
    auto paired_micro = [&](const PSub& q, int i, int dir) {
        const int64_t po = q.poff + i;
        const int j0 = P.p_j0[po], jc = P.p_cnt[po];
        const int li = P.vlev[FC.goff + i];
        const float* of = fbase + q.ofoff;
        const float* os = sbase + q.ofoff * D;
        const int onv = q.onv;
        float2 mic = bc2(0.f);
        for (int j = j0; j < j0 + jc; ++j) {
            const float uj0 = P.vuf[q.ogo + j], uj1 = P.vuf[P.PG + q.ogo + j];
            const float sc_ = merge_scale<D, float>(li, P.vlev[q.ogo + j]);
            const float2 g = make_float2(of[j], of[onv + j]);
            const float2 t0_ = make_float2(os[j], os[onv + j]);
            const float2 t1_ = make_float2(os[2 * onv + j], os[3 * onv + j]);
            const float ndx0 = q.dxo0 - uj0 * adt;
            const float ndx1 = q.dxo1 - uj1 * adt;
            const float2 nsdx = fma2(bc2(ndx1), t1_, mul2(bc2(ndx0), t0_));
            const float2 thn = pp_theta2(g, t0_, t1_, q.ods0, q.ods1);
            const float2 m = mul2(fma2(thn, nsdx, g), bc2(dir == 0 ? uj0 : uj1));
            mic = fma2(m, bc2(sc_), mic);
        }
        return mic;
    };
    // accM: the part of acc whose moments are the macro flux on this cell's grid (all but the
    // paired sub-faces' micro fluxes)
    float2 accM_last[VPT];
    auto gather_inner = [&](int i, const float4& V, float2& f2, float2& acc, float2& accM) {
        const float u0 = V.x, u1 = V.y;
        f2 = make_float2(fc[i], fc[nv + i]);
        const float2 s0 = make_float2(scl[i], scl[nv + i]);
        const float2 s1 = make_float2(scl[2 * nv + i], scl[3 * nv + i]);
        float2 g2[D][2], t0[D][2], t1[D][2];
        int so[D], si[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const bool pos = (d == 0 ? u0 : u1) > 0.f;
            so[d] = 2 * d + (pos ? 1 : 0);
            si[d] = 2 * d + (pos ? 0 : 1);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                // a side with one sub-face reads that one twice (in flight together; unused); a
                // paired sub-face's loads are its runs' (below)
                const PSub& qq = psub[si[d]][k < pcnt[si[d]] ? k : 0];
                const int64_t no = qq.ofoff;
                const int ii = (INNER == 1 || qq.pair < 0) ? i : 0;
                const float* of = fbase + no;
                const float* os = sbase + no * D;
                g2[d][k] = make_float2(of[ii], of[nv + ii]);
                t0[d][k] = make_float2(os[ii], os[nv + ii]);
                t1[d][k] = make_float2(os[2 * nv + ii], os[3 * nv + ii]);
            }
        }
        const float2 th = pp_theta2(f2, s0, s1, ds0, ds1);
        acc = bc2(0.f);
        accM = bc2(0.f);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const float ud = d == 0 ? u0 : u1;
            // outgoing through the side the velocity points at: the own reconstruction
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (k >= pcnt[so[d]]) break;
                const PSub& q = psub[so[d]][k];
                const float dx0 = q.dxm0 - u0 * adt;
                const float dx1 = q.dxm1 - u1 * adt;
                const float2 sdx = fma2(bc2(dx1), s1, mul2(bc2(dx0), s0));
                const float2 mo = mul2(fma2(th, sdx, f2), bc2(ud));
                acc = fma2(bc2(q.sa), mo, acc);
                accM = fma2(bc2(q.sa), mo, accM);
            }
            // incoming through the opposite side: the neighbours' reconstructions
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (k >= pcnt[si[d]]) break;
                const PSub& q = psub[si[d]][k];
                if constexpr (INNER == 2) {
                    if (q.pair >= 0) {
                        acc = fma2(bc2(q.sa), paired_micro(q, i, d), acc);
                        continue;
                    }
                }
                const float ndx0 = q.dxo0 - u0 * adt;
                const float ndx1 = q.dxo1 - u1 * adt;
                const float2 nsdx = fma2(bc2(ndx1), t1[d][k], mul2(bc2(ndx0), t0[d][k]));
                const float2 thn = pp_theta2(g2[d][k], t0[d][k], t1[d][k], q.ods0, q.ods1);
                const float2 mi = mul2(fma2(thn, nsdx, g2[d][k]), bc2(ud));
                acc = fma2(bc2(q.sa), mi, acc);
                accM = fma2(bc2(q.sa), mi, accM);
            }
        }
    };
    // the convected f, and the macro flux (CAIDVM) with the moments of the convected f (CAIDVM
    // marching) or of f (Euler) as the pairs (flux, f) in one set of packed sums
    auto finish = [&](int i, const float4& V, const float2& f2, const float2& acc, const float2& accM) {
        const float u0 = V.x, u1 = V.y, wi = V.z;
        const float2 fs = fma2(bc2(s_dt), acc, f2);
        fst[i] = fs;
        const float2 mf = march_caidvm ? fs : f2;
        const float2 H = make_float2(caidvm ? accM.x : 0.f, mf.x);
        const float2 B = make_float2(caidvm ? accM.y : 0.f, mf.y);
        float u2 = u0 * u0;
        u2 += u1 * u1;
        const float2 a0 = mul2(bc2(wi), H);
        m0 = add2(m0, a0);
        m1 = fma2(bc2(u0), a0, m1);
        m2 = fma2(bc2(u1), a0, m2);
        mE = fma2(bc2(0.5f * wi), fma2(bc2(u2), H, B), mE);
    };
    for (int i0 = threadIdx.x; i0 < nv; i0 += VPT * NT) {
        int iv[VPT];
        float4 V[VPT];
        float2 f2[VPT], acc[VPT];
#pragma unroll
        for (int v = 0; v < VPT; ++v) {
            iv[v] = i0 + v * NT;
            if (iv[v] >= nv) iv[v] = i0;    // a valid index for the loads; not finished
            V[v] = vel(iv[v]);
        }
#pragma unroll
        for (int v = 0; v < VPT; ++v) {
            if constexpr (INNER) gather_inner(iv[v], V[v], f2[v], acc[v], accM_last[v]);
            else { gather(iv[v], V[v], f2[v], acc[v]); accM_last[v] = acc[v]; }
        }
#pragma unroll
        for (int v = 0; v < VPT; ++v)
            if (v == 0 || i0 + v * NT < nv) finish(iv[v], V[v], f2[v], acc[v], accM_last[v]);
    }
    if constexpr (INNER == 2) {
        // the macro flux of the paired sub-faces on the neighbour's grid: the moments of its
        // micro fluxes at the velocities that leave it towards this cell, with its weights
        if (caidvm) {
#pragma unroll
            for (int sd = 0; sd < 4; ++sd) {
                const int d = sd >> 1;
                const bool plus = sd & 1;
                for (int k = 0; k < pcnt[sd]; ++k) {
                    const PSub& q = psub[sd][k];
                    if (q.pair < 0) continue;
                    const float* of = fbase + q.ofoff;
                    const float* os = sbase + q.ofoff * D;
                    const int onv = q.onv;
                    for (int j = threadIdx.x; j < onv; j += NT) {
                        const float uj0 = P.vuf[q.ogo + j], uj1 = P.vuf[P.PG + q.ogo + j];
                        const float ud = d == 0 ? uj0 : uj1;
                        if (plus ? !(ud < 0.f) : !(ud > 0.f)) continue;   // not towards this cell
                        const float2 g = make_float2(of[j], of[onv + j]);
                        const float2 t0_ = make_float2(os[j], os[onv + j]);
                        const float2 t1_ = make_float2(os[2 * onv + j], os[3 * onv + j]);
                        const float ndx0 = q.dxo0 - uj0 * adt;
                        const float ndx1 = q.dxo1 - uj1 * adt;
                        const float2 nsdx = fma2(bc2(ndx1), t1_, mul2(bc2(ndx0), t0_));
                        const float2 thn = pp_theta2(g, t0_, t1_, q.ods0, q.ods1);
                        const float2 m = mul2(fma2(thn, nsdx, g), bc2(ud));
                        const float wj = P.vwf[q.ogo + j] * q.sa;
                        float u2 = uj0 * uj0;
                        u2 += uj1 * uj1;
                        const float a0 = wj * m.x;
                        m0.x += a0;
                        m1.x += uj0 * a0;
                        m2.x += uj1 * a0;
                        mE.x += 0.5f * wj * (u2 * m.x + m.y);
                    }
                }
            }
        }
    }
    double qv[D];
    {
        double red[2 * (D + 2)];
        float hi[2 * (D + 2)] = {m0.x, m1.x, m2.x, mE.x, m0.y, m1.y, m2.y, mE.y};
        float lo[2 * (D + 2)] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        block_sum_ff<2 * (D + 2), NT>(hi, lo, red, sred);
        cell_constants<D, 2, float, NT, 4>(P, cell, slot, PP, dt, FC.invV, red, sscal, sc, &T4[0].x, FC.gid);
    }
    const float prec = sc[C_PREC], pren = sc[C_PREN], bfc = sc[C_BFC], bfn = sc[C_BFN];
    // ---- 3. conservation correction f += M(prim_c) - M(prim) (CAIDVM marching) and q -------
    {
        float2 q2 = bc2(0.f);
#pragma unroll 4
        for (int i = threadIdx.x; i < nv; i += NT) {
            const int ix = vxa[i], iy = vxb[i];
            const float4 ta = T4[ix], tb = T4[MA + iy];
            float2 fv;
            if (march_caidvm) {
                float mc = prec;
                mc *= ta.x;
                mc *= tb.x;
                float mn = pren;
                mn *= ta.y;
                mn *= tb.y;
                const float2 fs = fst[i];
                fv = make_float2(fs.x + (mc - mn), fs.y + (mc * bfc - mn * bfn));
                fst[i] = fv;
            } else {
                fv = make_float2(fc[i], fc[nv + i]);   // Euler: q of f before convection
            }
            const float c0 = ta.w, c1 = tb.w;   // (u_d - U_hi) - U_lo from the table
            float c2 = c0 * c0;
            c2 += c1 * c1;
            const float hb = c2 * fv.x + fv.y;
            q2 = fma2(mul2(bc2(vwt[i]), make_float2(c0, c1)), bc2(hb), q2);
        }
        float hi[D] = {q2.x, q2.y}, lo[D] = {0.f, 0.f};
        block_sum_ff<D, NT>(hi, lo, qv, sred);
        if (threadIdx.x == 0)
            for (int d = 0; d < D; ++d) sc[C_QA + d] = (float)(0.5 * qv[d]);
        __syncthreads();
    }
    // ---- 4. Shakhov g+ (shakhov_part_2D2F) and the implicit relaxation --------------------
    {
        const float r1 = sc[C_R1], r2 = sc[C_R2], sk = sc[C_SK], lc = sc[C_LC];
        const float Kk = (float)PP.K;
        const float qa0 = sc[C_QA], qa1 = sc[C_QA + 1];
        float* fo = (float*)P.f_out + FC.foff;
#pragma unroll 4
        for (int i = threadIdx.x; i < nv; i += NT) {
            const int ix = vxa[i], iy = vxb[i];
            const float4 ta = T4[ix], tb = T4[MA + iy];
            float mc = prec;
            mc *= ta.x;
            mc *= tb.x;
            const float c0 = ta.w, c1 = tb.w;   // (u_d - U_hi) - U_lo from the table
            float c2 = c0 * c0;
            c2 += c1 * c1;
            float cq = c0 * qa0;
            cq += c1 * qa1;
            const float mb = mc * bfc;
            const float pol = 2.f * lc * c2 + Kk;
            const float2 gp = make_float2(mc + sk * cq * (pol - 5.f) * mc, mb + sk * cq * (pol - 3.f) * mb);
            const float2 fn = fma2(bc2(r2), gp, mul2(fst[i], bc2(r1)));
            fo[i] = fn.x;
            fo[nv + i] = fn.y;
        }
    }
    cell_outputs<D>(P, cell, fcx, step, PP.check, sscal, qv);
}

// Flux + collision of the fluid cells.  Two schedules share this one function, so the
// arithmetic of a cell compiles once and gives the same bits under either:
//  * counter == nullptr: one CTA per fluid cell (cell = blockIdx.x);
//  * persistent: `gridDim.x` resident CTAs take cells from the work counter (in `order`,
//    when given), so a batch of uneven problems keeps every SM busy to the end of the
//    sub-step.  The counter must be zero at launch.
// MB: resident 256-thread-CTA equivalents the registers allow (0: 4 in FP32, 2 in FP64)
template <int D, int NDF, typename T, bool FG, int NT, bool PPIB = false, int MB = 0>
__global__ void __launch_bounds__(NT, (MB ? MB : (sizeof(T) == 4 ? 4 : 2)) * (BLOCK / NT)) flux_collide_kernel(Dev P, int* counter,
                                                                                             const int32_t* order, int n) {
    __shared__ int item;
    int it = blockIdx.x;
    for (;;) {
        if (counter) {
            if (threadIdx.x == 0) item = atomicAdd(counter, 1);
            __syncthreads();
            it = item;
            __syncthreads();
        }
        if (it >= n) break;
        flux_collide_cell<D, NDF, T, FG, NT, false, PPIB>(P, order ? order[it] : it);
        if (!counter) break;
        __syncthreads();
    }
}

// Flux + collision of the listed regular fluid cells, one CTA each (the generic cell's regular
// branch; the 2D mixed form under CAIDVM or Euler marching takes flux_packed_kernel instead).
template <int D, int NDF, typename T, bool FG, int NT>
__global__ void __launch_bounds__(NT, (sizeof(T) == 4 ? 4 : 2) * (BLOCK / NT)) flux_regular_kernel(Dev P,
                                                                                             const int32_t* list) {
    flux_collide_cell<D, NDF, T, FG, NT, true>(P, list[blockIdx.x]);
}
// VPT velocity cells per thread and pass of the gather (their loads in flight together);
// more registers, so fewer resident CTAs
// Programmatic dependent launch (sm_90+) of the packed forms one after another on a stream: a
// kernel launched with programmatic stream serialization may start once every CTA of the kernel
// before it has executed launch_dependents (here at its start), so its CTAs fill the SMs the
// other's last wave frees; the packed forms read nothing another writes, and each CTA waits at
// its end until the kernel before has completed, so that the stream's next operation, ordered
// after the last kernel, finds them all complete (both are no-ops under an ordinary launch).
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
template <int NT, int VPT, bool R2>
__global__ void __launch_bounds__(NT, (R2 ? 3 : (VPT == 1 ? 4 : KG_PACKED_MINB)) * (BLOCK / NT)) flux_packed_kernel(Dev P, const int32_t* list) {
    pdl_trigger();
    flux_regular_packed<NT, VPT, R2>(P, list[blockIdx.x]);
    pdl_wait();
}
// the cells of packed_inner_ok, one CTA each (PAIRED: some sub-face to another velocity grid)
template <int NT, bool PAIRED>
__global__ void __launch_bounds__(NT, 3 * (BLOCK / NT)) flux_packed_inner_kernel(Dev P, const int32_t* list) {
    pdl_trigger();
    flux_regular_packed<NT, 1, false, PAIRED ? 2 : 1>(P, list[blockIdx.x]);
    pdl_wait();
}

// Per fluid-list entry: 1 when the packed kernel's INNER form takes the cell (not regular; every
// incidence an inner face to a fluid cell on its own velocity grid, leaving through the side its
// face points at; one or two sub-faces on each of the four sides), 2 when it does so with some
// neighbour on another grid, else 0.
__global__ void packed_inner_ok_kernel(Dev P, int n, uint8_t* out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    uint8_t ok = 0;
    bool paired = false;
    if (!P.fluid_reg[q]) {
        const FluxCell& FC = P.fcrec[q];
        int cnt[4] = {0, 0, 0, 0};
        ok = FC.ninc > 0;
        for (int e = 0; e < FC.ninc && ok; ++e) {
            const Incidence& a = P.inc[FC.inc0 + e];
            const int d = a.dir;
            ok = a.kind == INC_INNER && d >= 0 && d < 2 && a.orient_f * a.dxm_f[d] < 0.f;
            paired = paired || a.pair >= 0;
            if (ok) {
                const int sd = 2 * d + (a.dxm_f[d] > 0.f ? 1 : 0);
                ok = ++cnt[sd] <= 2;
            }
        }
        for (int sd = 0; sd < 4 && ok; ++sd) ok = cnt[sd] >= 1;
    }
    out[q] = ok ? (paired ? 2 : 1) : 0;
}
cudaError_t launch_packed_inner_ok(const Dev& P, int n, uint8_t* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    packed_inner_ok_kernel<<<(n + 255) / 256, 256, 0, s>>>(P, n, out);
    return cudaGetLastError();
}

// update_macro_slope! (Flux/Slope.jl:1022-1036): sw[:, dir] = calc_w0(midpoint, sdf[:, :, dir],
// weight) for the fluid-list cells [fbegin, fbegin + gridDim.x), one CTA each; out holds
// dim x (dim+2) doubles per data item from dbase on (the column-major memory of PsData.sw).
// Not part of a step: it reads the slopes the last step left, at a host sync point.
template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK) macro_slope_kernel(Dev P, int fbegin, int dbase, double* out) {
    using A = typename Arith<T>::type;
    constexpr int N = D * (D + 2);
    __shared__ double sred[N * (BLOCK / 32)];
    const int cell = P.fluid_cells[fbegin + blockIdx.x];
    const VGridView g = grid_view(P, cell);
    const int nv = g.nv;
    const T* s = (const T*)P.sdf + P.foff[cell] * D;
    const A* VU = vel<A>(P);
    const A* VW = wts<A>(P) + g.goff;
    KSum<A> m[N];
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        A u[D], u2 = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) { u[d] = VU[(int64_t)d * P.PG + g.goff + i]; u2 += u[d] * u[d]; }
        const A wi = VW[i];
#pragma unroll
        for (int dir = 0; dir < D; ++dir) {
            const A s0 = (A)s[((int64_t)dir * NDF) * nv + i];
            m[dir * (D + 2)].add(wi * s0);
#pragma unroll
            for (int d = 0; d < D; ++d) m[dir * (D + 2) + 1 + d].add(wi * u[d] * s0);
            if (NDF == 2) {
                const A s1 = (A)s[((int64_t)dir * NDF + NDF - 1) * nv + i];
                m[dir * (D + 2) + D + 1].add((A)0.5 * wi * (u2 * s0 + s1));
            } else {
                m[dir * (D + 2) + D + 1].add((A)0.5 * wi * u2 * s0);
            }
        }
    }
    double r[N];
    block_sum_ks<N>(m, r, sred);
#pragma unroll
    for (int e = 0; e < N; ++e)
        if (threadIdx.x == e) out[(int64_t)(cell - dbase) * N + e] = r[e];
}

// ---- physical-space criterion (update_criterion!, Physical_space/AMR.jl:256-284) --------
// Julia's max of floats propagates NaN (fmax does not)
__device__ __forceinline__ double jl_max(double a, double b) { return (a != a || b != b) ? a + b : (a > b ? a : b); }

// lohner_value (Physical_space/Criteria.jl:24-30)
__device__ __forceinline__ double lohner_value(double l, double c, double r, double dsL, double dsR, double eps) {
    const double scale = dsR * fabs(l) + (dsL + dsR) * fabs(c) + dsL * fabs(r);
    if (scale < 1e-4 * (dsL < dsR ? dsL : dsR)) return 0.0;            // PS_LOHNER_ABS_FLOOR
    const double denom = dsR * fabs(l - c) + dsL * fabs(r - c) + eps * scale;
    if (denom <= 0.0) return 0.0;
    return fabs(dsR * l - (dsL + dsR) * c + dsL * r) / denom;
}
// primitive_amplitude_ok (Criteria.jl:32-36)
__device__ __forceinline__ bool primitive_amplitude_ok(double l, double c, double r) {
    const double jump = jl_max(fabs(l - c), fabs(r - c));
    const double scale = jl_max(fabs(c), 1e-4);
    return jump >= 1e-3 * scale;                                        // PS_PRIMITIVE_REL_JUMP_FLOOR
}
// velocity_slope and vorticity (Criteria.jl:38-52): sw is [dir][component] (PsData.sw memory)
template <int D>
__device__ __forceinline__ double velocity_slope(const double* sw, const double* prim, int c, int dir) {
    return (sw[dir * (D + 2) + c] - prim[c] * sw[dir * (D + 2)]) / prim[0];
}
template <int D>
__device__ __forceinline__ double vorticity(const double* sw, const double* prim) {
    if (D == 2) return velocity_slope<D>(sw, prim, 1, 1) - velocity_slope<D>(sw, prim, 2, 0);
    const double c1 = velocity_slope<D>(sw, prim, 2, 2) - velocity_slope<D>(sw, prim, 3, 1);
    const double c2 = velocity_slope<D>(sw, prim, 3, 0) - velocity_slope<D>(sw, prim, 1, 2);
    const double c3 = velocity_slope<D>(sw, prim, 1, 1) - velocity_slope<D>(sw, prim, 2, 0);
    return sqrt(c1 * c1 + c2 * c2 + c3 * c3);
}
// velocity_scale, vorticity_amplitude_ok (Criteria.jl:54-66)
template <int D>
__device__ __forceinline__ bool vorticity_amplitude_ok(double l, double c, double r, const double* prim, double h) {
    double speed2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) speed2 += prim[1 + d] * prim[1 + d];
    const double lambda = jl_max(fabs(prim[D + 1]), JL_EPS);
    const double vscale = jl_max(sqrt(speed2), 1.0 / sqrt(lambda));
    const double omega = jl_max(fabs(l), jl_max(fabs(c), fabs(r)));
    return omega * h >= 2e-2 * vscale;                                  // PS_VORTICITY_JUMP_FLOOR
}

// update_Lohner_inner_ps! (Criteria.jl:95-158) of the fluid cells [fbegin, fbegin + n), one
// thread each, in FP64; sw and loh are indexed by data index - dbase, (dim+2) x dim doubles
// per item (the column-major memory of PsData.sw / PsData.lohner).
template <int D>
__global__ void criterion_kernel(Dev P, int fbegin, int n, int dbase, const double* sw, double* loh) {
    constexpr int NW = D + 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int fcx = fbegin + q;
    const int cell = P.fluid_cells[fcx];
    const double* swc = sw + (int64_t)(cell - dbase) * NW * D;
    double* lo = loh + (int64_t)(cell - dbase) * NW * D;
    const double* pc = P.prim + (int64_t)cell * MAXW;
    const double* mc = P.dmid + (int64_t)cell * MAXD;
    const double gamma = P.probs[P.dprob[cell]].gamma;
    const double omega_c = vorticity<D>(swc, pc);
    for (int dir = 0; dir < D; ++dir) {
        const CritOp op = P.crit_ops[(int64_t)fcx * D + dir];
        double* row = lo + dir * NW;
        if (op.kind == 0) {
#pragma unroll
            for (int j = 0; j < NW; ++j) row[j] = 0.0;
            continue;
        }
        // each side: the mean of its neighbours' w and sw, a coarser side's w corrected along
        // the transverse directions with its sw; then its primitives and vorticity
        double pside[2][NW], omega[2];
        for (int side = 0; side < 2; ++side) {
            const int list = side == 0 ? op.listA : op.listB, nl = side == 0 ? op.cntA : op.cntB;
            double ws[NW], sws[NW * D];
#pragma unroll
            for (int j = 0; j < NW; ++j) ws[j] = 0.0;
            for (int e = 0; e < NW * D; ++e) sws[e] = 0.0;
            for (int k = 0; k < nl; ++k) {
                const int nb = P.crit_nbr[list + k];
                // a SolidNeighbor keeps w = sw = 0 (Immersed_boundary.jl:300-302, 481-482): its
                // side's density is 0 and its velocities and lambda NaN, so only the density
                // row of that direction can be nonzero
                if (nb < 0) continue;
                const double* wn = P.w + (int64_t)nb * MAXW;
                const double* swn = sw + (int64_t)(nb - dbase) * NW * D;
#pragma unroll
                for (int j = 0; j < NW; ++j) ws[j] += wn[j];
                for (int e = 0; e < NW * D; ++e) sws[e] += swn[e];
            }
            if ((side == 0 ? op.coarseA : op.coarseB) && P.crit_nbr[list] >= 0) {
                const int nb = P.crit_nbr[list];
                const double* nm = P.dmid + (int64_t)nb * MAXD;
                const double* swn = sw + (int64_t)(nb - dbase) * NW * D;
                for (int t = 0; t < D; ++t) {
                    if (t == dir) continue;                    // FAT: the transverse directions
                    const double dx = mc[t] - nm[t];
#pragma unroll
                    for (int j = 0; j < NW; ++j) ws[j] += dx * swn[t * NW + j];
                }
            }
#pragma unroll
            for (int j = 0; j < NW; ++j) ws[j] /= nl;
            for (int e = 0; e < NW * D; ++e) sws[e] /= nl;
            get_prim<D>(ws, gamma, pside[side]);
            omega[side] = vorticity<D>(sws, pside[side]);
        }
        const double dsL = op.dsA, dsR = op.dsB;
        const bool use_vort = vorticity_amplitude_ok<D>(omega[0], omega_c, omega[1], pc, dsL > dsR ? dsL : dsR);
        const double eps_l = 0.2 * P.dds[(int64_t)cell * MAXD + dir];
#pragma unroll
        for (int j = 0; j < NW; ++j) {
            if (j == 1)
                row[j] = use_vort ? lohner_value(omega[0], omega_c, omega[1], dsL, dsR, eps_l) : 0.0;
            else
                row[j] = primitive_amplitude_ok(pside[0][j], pc[j], pside[1][j])
                             ? lohner_value(pside[0][j], pc[j], pside[1][j], dsL, dsR, eps_l) : 0.0;
        }
    }
}

// ps_sensor (Criteria.jl:14-21): max over directions of the density and last rows
template <int D>
__device__ __forceinline__ double ps_sensor(const double* lo) {
    double v = 0.0;
    for (int dir = 0; dir < D; ++dir) v = jl_max(v, jl_max(lo[dir * (D + 2)], lo[dir * (D + 2) + D + 1]));
    return v;
}

// apply_amr_buffer! (Physical_space/AMR.jl:286-330): a cell at or below the threshold whose
// neighbour (any non-boundary side, fluid cells only) is above it gets lohner = 2 threshold;
// decide on loh, write out.
template <int D>
__global__ void criterion_buffer_kernel(Dev P, int fbegin, int n, int dbase, double thr, const double* loh,
                                        double* out) {
    constexpr int NW = D + 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int fcx = fbegin + q;
    const int cell = P.fluid_cells[fcx];
    const double* lo = loh + (int64_t)(cell - dbase) * NW * D;
    bool flagged = false;
    if (!(ps_sensor<D>(lo) > thr)) {
        for (int dir = 0; dir < D && !flagged; ++dir) {
            const CritOp op = P.crit_ops[(int64_t)fcx * D + dir];
            for (int side = 0; side < 2 && !flagged; ++side) {
                const int list = side == 0 ? op.listA : op.listB, nl = side == 0 ? op.cntA : op.cntB;
                for (int k = 0; k < nl; ++k) {
                    const int nb = P.crit_nbr[list + k];
                    if (nb < 0 || P.dbe[nb] < 0) continue;
                    if (ps_sensor<D>(loh + (int64_t)(nb - dbase) * NW * D) > thr) { flagged = true; break; }
                }
            }
        }
    }
    double* o = out + (int64_t)(cell - dbase) * NW * D;
    for (int e = 0; e < NW * D; ++e) o[e] = flagged ? 2.0 * thr : lo[e];
}

// Per problem (one CTA each): Σ of the per-cell residual terms when the step is a check
// step (residual_check!, Solver/Finalize.jl:5-11), then the problem's step counter
// advances (iterate!, Theory/Iterate.jl:10).  Fixed summation order: deterministic.
__global__ void __launch_bounds__(BLOCK) residual_kernel(Dev P, const int32_t* live, double* out) {
    __shared__ double sred[2 * MAXW * (BLOCK / 32)];
    const int slot = live[blockIdx.x];
    const ProbParams& PP = P.probs[slot];
    const int64_t step = P.prob_step[slot];
    const bool chk = (step % PP.check) == 0;
    if (chk) {
        double v[2 * MAXW];
#pragma unroll
        for (int q = 0; q < 2 * MAXW; ++q) v[q] = 0.0;
        for (int c = PP.fluid_begin + threadIdx.x; c < PP.fluid_end; c += BLOCK)
#pragma unroll
            for (int q = 0; q < 2 * MAXW; ++q) v[q] += P.cell_res[(int64_t)c * 2 * MAXW + q];
        block_sum<2 * MAXW>(v, sred);
        if (threadIdx.x == 0) {
            double* o = out + (int64_t)slot * RES_STRIDE;
#pragma unroll
            for (int q = 0; q < 2 * MAXW; ++q) o[q] = v[q];
            o[2 * MAXW] = (double)step;
            o[2 * MAXW + 1] = 1.0;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) P.prob_step[slot] = step + 1;
}

// ---- launchers ------------------------------------------------------------------
// ---- velocity-space adaptation flags (vs_refine! / vs_coarsen!, Velocity_space/AMR.jl:26-118)
// Block maximum of N doubles (every thread sees the result); sred: N * (BLOCK/32) doubles.
template <int N>
__device__ __forceinline__ void block_max(double (&v)[N], double* sred) {
    constexpr int NWARP = BLOCK / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int e = 0; e < N; ++e) {
        double x = v[e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
        v[e] = x;
    }
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int e = 0; e < N; ++e) sred[e * NWARP + wid] = v[e];
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < N; ++e) {
        double x = sred[e * NWARP];
        for (int q = 1; q < NWARP; ++q) x = fmax(x, sred[e * NWARP + q]);
        v[e] = x;
    }
    __syncthreads();
}

// vs_resolution (Velocity_space/AMR.jl:153-166) of the cells [c0, c0 + gridDim.x): the largest
// df entry and the largest h|U-u|^2 + b (3D: f|U-u|^2) of each, into out[2 * (cell - c0)]
template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK) vs_resolution_kernel(Dev P, int c0, double* out) {
    __shared__ double sred[2 * (BLOCK / 32)];
    const int cell = c0 + blockIdx.x;
    const VGridView g = grid_view(P, cell);
    const int nv = g.nv;
    const T* fc = (const T*)P.f_in + P.foff[cell];
    const double* U = P.prim + (int64_t)cell * MAXW + 1;
    double m[2] = {-INFINITY, -INFINITY};
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        double c2 = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) { const double x = U[d] - P.vu[(int64_t)d * P.PG + g.goff + i]; c2 += x * x; }
        const double h = (double)fc[i];
        m[0] = fmax(m[0], h);
        if (NDF == 2) {
            const double b = (double)fc[nv + i];
            m[0] = fmax(m[0], b);
            m[1] = fmax(m[1], h * c2 + b);
        } else {
            m[1] = fmax(m[1], h * c2);
        }
    }
    block_max<2>(m, sred);
    if (threadIdx.x == 0) { out[2 * blockIdx.x] = m[0]; out[2 * blockIdx.x + 1] = m[1]; }
}


// _lohner_ratio (Velocity_space/Criteria.jl:221-227)
__device__ __forceinline__ double vs_lohner_ratio(double L, double C, double R, double dsL, double dsR, double scale) {
    const double num = fabs(dsR * L - (dsL + dsR) * C + dsL * R);
    const double den = dsR * fabs(L - C) + dsL * fabs(R - C) +
                       1e-2 * (dsR * fabs(L) + (dsL + dsR) * fabs(C) + dsL * fabs(R)) + 1e-3 * scale * (dsL + dsR);
    return den > 0 ? num / den : 0.0;
}

// The flags of vs_refine! / vs_coarsen! for the cells [c0, c0 + gridDim.x), one CTA each, in
// FP64: the criterion distribution and contribution flags (_criterion_cell!,
// local_/global_contribution_*_flag, Criteria.jl:18-78) and the Löhner indicator
// (vs_lohner_indicator, Criteria.jl:253-283) over the face-neighbour table.
template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK) vs_flags_kernel(Dev P, int c0, VsFlagArgs A) {
    __shared__ double sred[2 * (BLOCK / 32)];
    const int cell = c0 + blockIdx.x;
    const VGridView g = grid_view(P, cell);
    const int nv = g.nv;
    const int64_t fo = P.foff[cell];
    const T* fc = (const T*)P.f_in + fo;
    const T* sc = (const T*)P.sdf + fo * D;
    const double* wc = P.w + (int64_t)cell * MAXW;
    const double* U = P.prim + (int64_t)cell * MAXW + 1;
    const double* ds = P.dds + (int64_t)cell * MAXD;
    const int32_t* nb = A.nbr + (g.goff) * 2 * D;
    const int8_t* lev = P.vlev + g.goff;
    // vs_lohner_scales: the largest |h| and |b| of the cell
    double s[2] = {0.0, 0.0};
    if (A.lohner) {
        for (int i = threadIdx.x; i < nv; i += BLOCK) {
            s[0] = fmax(s[0], fabs((double)fc[i]));
            if (NDF == 2) s[1] = fmax(s[1], fabs((double)fc[nv + i]));
        }
        block_max<2>(s, sred);
    }
    double U2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) U2 += U[d] * U[d];
    const double den = wc[D + 1] - 0.5 * wc[0] * U2;
    const double nch = (double)(1 << D);
    const int64_t row = (fo - A.row0) / NDF;
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        double cdf[NDF];
#pragma unroll
        for (int k = 0; k < NDF; ++k) {
            double mm = 0.0;
#pragma unroll
            for (int d = 0; d < D; ++d) mm = fmax(mm, fabs((double)sc[((int64_t)d * NDF + k) * nv + i] * ds[d]));
            cdf[k] = (double)fc[(int64_t)k * nv + i] + mm;
        }
        double S = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) { const double x = U[d] - P.vu[(int64_t)d * P.PG + g.goff + i]; S += x * x; }
        const double wt = P.vw[g.goff + i];
        const double en = NDF == 2 ? 0.5 * (S * cdf[0] + cdf[NDF - 1]) * wt : 0.5 * S * cdf[0] * wt;
        const double rho = cdf[0] * wt;
        const bool loc_ref = fmax(fabs(en) / den, rho / wc[0]) > A.c_local;
        const bool loc_coa = fmax(en / den, rho / wc[0]) < A.c_local / nch;
        const bool glo_ref = rho > A.c_global * A.dens_res || en > A.en_res * A.c_global;
        const bool glo_coa = rho < A.c_global * A.dens_res / nch && en < A.en_res * A.c_global / nch;
        double e = 0.0;
        if (A.lohner) {
            const int li = lev[i];
            const double h0 = (double)fc[i];
            const double b0 = NDF == 2 ? (double)fc[nv + i] : 0.0;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const double hi = A.hf[d] * (double)(1 << (A.maxlevel - li));
                const int Ln = nb[(int64_t)i * 2 * D + 2 * d], Rn = nb[(int64_t)i * 2 * D + 2 * d + 1];
                const double dsL = Ln < 0 ? hi : 0.5 * (hi + A.hf[d] * (double)(1 << (A.maxlevel - lev[Ln])));
                const double dsR = Rn < 0 ? hi : 0.5 * (hi + A.hf[d] * (double)(1 << (A.maxlevel - lev[Rn])));
                const double hL = Ln < 0 ? 0.0 : (double)fc[Ln], hR = Rn < 0 ? 0.0 : (double)fc[Rn];
                e = fmax(e, vs_lohner_ratio(hL, h0, hR, dsL, dsR, s[0]));
                if (NDF == 2) {
                    const double bL = Ln < 0 ? 0.0 : (double)fc[nv + Ln], bR = Rn < 0 ? 0.0 : (double)fc[nv + Rn];
                    e = fmax(e, vs_lohner_ratio(bL, b0, bR, dsL, dsR, s[1]));
                }
            }
        }
        const bool refine = lev[i] < A.maxlevel && (A.lohner ? (e > A.tau_l || loc_ref) : (loc_ref || glo_ref));
        const bool coarsen = A.lohner ? (e < A.tau_c && loc_coa) : (loc_coa && glo_coa);
        A.flags[row + i] = (uint8_t)((refine ? 1 : 0) | (coarsen ? 2 : 0));
        if (A.eta) A.eta[row + i] = e;
    }
}

// ---- physical-space adaptation (ps_replace!, Physical_space/AMR.jl:633-703) ----------
// One CTA per cell of the adapted mesh (layout P, state written into P.f_in / P.sdf / P.w /
// P.prim / P.qf) from the pools of the previous mesh (V).  Arithmetic in the form's precision
// (the refinement limiter and the merge sums); w of a refined cell is its calc_w0 (block
// reduction), prim = get_prim of w.
template <typename T> struct AdaptView {
    const AdaptRec* recs;
    const T* f;             // previous f (the buffer the next step would have read)
    const T* sdf;           // previous slopes (recomputed from that f)
    const double* w;
    const double* prim;
    const double* qf;
    const int32_t* runs;    // (j0, count) pairs of the coarsening merges
    const int8_t* lev;      // velocity levels of the children's grids
};

template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK) adapt_kernel(Dev P, AdaptView<T> V) {
    using A = typename Arith<T>::type;
    __shared__ double sred[(D + 2) * (BLOCK / 32)];
    const AdaptRec& R = V.recs[blockIdx.x];
    const int cell = R.cell;
    const VGridView g = grid_view(P, cell);
    const int nv = g.nv;
    const int64_t fo = P.foff[cell];
    T* fn = (T*)P.f_in + fo;
    T* sn = (T*)P.sdf + fo * D;
    double* wn = P.w + (int64_t)cell * MAXW;
    double* pn = P.prim + (int64_t)cell * MAXW;
    double* qn = P.qf + (int64_t)cell * MAXD;
    if (R.kind == KG_ADAPT_KEEP) {
        const T* fs = V.f + R.src_f[0];
        const T* ss = V.sdf + R.src_f[0] * D;
        for (int64_t a = threadIdx.x; a < (int64_t)NDF * nv; a += BLOCK) fn[a] = fs[a];
        for (int64_t a = threadIdx.x; a < (int64_t)D * NDF * nv; a += BLOCK) sn[a] = ss[a];
        const int64_t od = R.src_d[0];
        if (threadIdx.x < D + 2) {
            wn[threadIdx.x] = V.w[od * MAXW + threadIdx.x];
            pn[threadIdx.x] = V.prim[od * MAXW + threadIdx.x];
        }
        if (threadIdx.x < D) qn[threadIdx.x] = V.qf[od * MAXD + threadIdx.x];
        return;
    }
    if (R.kind == KG_ADAPT_VS) {
        // refine_grid_stream! / coarsen_grid_stream! (Velocity_space/Rebuild.jl:44-163): each
        // velocity cell of the new grid from the run of source cells it overlaps -- a coarser
        // source cell (refinement) copied, 2^dim finer siblings (coarsening) summed over 2^dim
        // (the same bits as their sum over 2^dim); slopes zero, w, prim and qf kept
        const T* fs = V.f + R.src_f[0];
        const int nvs = R.src_nv[0];
        for (int i = threadIdx.x; i < nv; i += BLOCK) {
            const int li = P.vlev[g.goff + i];
            int j0 = i, cnt = 1;
            if (R.run[0] >= 0) { j0 = V.runs[2 * (R.run[0] + i)]; cnt = V.runs[2 * (R.run[0] + i) + 1]; }
#pragma unroll
            for (int k = 0; k < NDF; ++k) {
                A acc = 0;
                for (int j = j0; j < j0 + cnt; ++j) {
                    const int sh = R.run[0] >= 0 ? D * ((int)V.lev[R.lev[0] + j] - li) : 0;
                    const A v = (A)fs[(int64_t)k * nvs + j];
                    acc += sh > 0 ? v / (A)(1 << sh) : v;
                }
                fn[(int64_t)k * nv + i] = (T)acc;
            }
        }
        for (int64_t a = threadIdx.x; a < (int64_t)D * NDF * nv; a += BLOCK) sn[a] = (T)0;
        const int64_t od = R.src_d[0];
        if (threadIdx.x < D + 2) {
            wn[threadIdx.x] = V.w[od * MAXW + threadIdx.x];
            pn[threadIdx.x] = V.prim[od * MAXW + threadIdx.x];
        }
        if (threadIdx.x < D) qn[threadIdx.x] = V.qf[od * MAXD + threadIdx.x];
        return;
    }
    if (R.kind == KG_ADAPT_REFINE) {
        const T* fs = V.f + R.src_f[0];
        const T* ss = V.sdf + R.src_f[0] * D;
        const A* VU = vel<A>(P);
        const A* VW = wts<A>(P) + g.goff;
        KSum<A> m[D + 2];
        for (int i = threadIdx.x; i < nv; i += BLOCK) {
            A fv[NDF];
#pragma unroll
            for (int k = 0; k < NDF; ++k) {
                A x = (A)fs[(int64_t)k * nv + i];
                A s[D];
#pragma unroll
                for (int d = 0; d < D; ++d) s[d] = (A)ss[((int64_t)d * NDF + k) * nv + i];
                double dsl[D];
#pragma unroll
                for (int d = 0; d < D; ++d) dsl[d] = R.ds[d];
                for (int l = 0; l < R.depth; ++l) {
                    // the child's ds and its offset 0.5 ds .* RMT[child] from the parent centre
                    A den = 0, dot = 0;
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        dsl[d] *= 0.5;
                        const A dd = (A)dsl[d];
                        den += dd * fabs(s[d]);
                        const A off = ((R.path[l] >> d) & 1) ? (A)0.5 * dd : -((A)0.5 * dd);
                        dot += s[d] * off;
                    }
                    den += (A)EPS_REF;
                    A th = fabs(x / den);
                    th = th < (A)1 ? th : (A)1;
                    x += th * dot;
                }
                fv[k] = x;
                fn[(int64_t)k * nv + i] = (T)x;
#pragma unroll
                for (int d = 0; d < D; ++d) sn[((int64_t)d * NDF + k) * nv + i] = ss[((int64_t)d * NDF + k) * nv + i];
            }
            A u[D];
#pragma unroll
            for (int d = 0; d < D; ++d) u[d] = VU[(int64_t)d * P.PG + g.goff + i];
            moments_add_a<D, NDF, A>(u, VW[i], fv, m);
        }
        double mw[D + 2];
        block_sum_ks<D + 2>(m, mw, sred);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int e = 0; e < D + 2; ++e) wn[e] = mw[e];
            get_prim<D>(mw, P.probs[P.dprob[cell]].gamma, pn);
#pragma unroll
            for (int d = 0; d < D; ++d) qn[d] = 0.0;
        }
        return;
    }
    // KG_ADAPT_COARSEN: vs_merge! of every child onto this grid (in child order), over 2^D
    const A inv_children = (A)1 / (A)(1 << D);
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        const int li = P.vlev[g.goff + i];
        A acc[(D + 1) * NDF];
#pragma unroll
        for (int q = 0; q < (D + 1) * NDF; ++q) acc[q] = 0;
        for (int c = 0; c < R.nsrc; ++c) {
            const T* fs = V.f + R.src_f[c];
            const T* ss = V.sdf + R.src_f[c] * D;
            const int nvc = R.src_nv[c];
            int j0 = i, cnt = 1;
            if (R.run[c] >= 0) { j0 = V.runs[2 * (R.run[c] + i)]; cnt = V.runs[2 * (R.run[c] + i) + 1]; }
            for (int j = j0; j < j0 + cnt; ++j) {
                const int sh = R.run[c] >= 0 ? D * ((int)V.lev[R.lev[c] + j] - li) : 0;
                const A div = sh > 0 ? (A)(1 << sh) : (A)1;
#pragma unroll
                for (int k = 0; k < NDF; ++k) {
                    const A v = (A)fs[(int64_t)k * nvc + j];
                    acc[k] += sh > 0 ? v / div : v;
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        const A sv = (A)ss[((int64_t)d * NDF + k) * nvc + j];
                        acc[NDF + d * NDF + k] += sh > 0 ? sv / div : sv;
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < NDF; ++k) {
            fn[(int64_t)k * nv + i] = (T)(acc[k] * inv_children);
#pragma unroll
            for (int d = 0; d < D; ++d) sn[((int64_t)d * NDF + k) * nv + i] = (T)(acc[NDF + d * NDF + k] * inv_children);
        }
    }
    if (threadIdx.x == 0) {
        double mw[D + 2];
#pragma unroll
        for (int e = 0; e < D + 2; ++e) {
            double s = 0.0;
            for (int c = 0; c < R.nsrc; ++c) s += V.w[(int64_t)R.src_d[c] * MAXW + e];
            mw[e] = s / (double)(1 << D);
            wn[e] = mw[e];
        }
        get_prim<D>(mw, P.probs[P.dprob[cell]].gamma, pn);
#pragma unroll
        for (int d = 0; d < D; ++d) qn[d] = 0.0;
    }
}

// ---- CIP_Marching: conservative I-projection and relaxation ------------------------------
// iterate!(CIP_Marching) (Theory/I-projection.jl:161-193) after the flux kernel, which leaves
// in f_out the convected f of every fluid cell, in w the conserved update, in prim prim_c and
// in qf the heat flux of the convected f.  One CTA per fluid cell:
//  1. conserved_I_porjection! (:144-158): W = w (2D2F: less the energy Σ ω f₂ / 2 of the second
//     distribution); solve_I_projection (:55-141) on f₁ -- the negative-value shave, then Newton
//     iterations on G(λ) = Σ ω f e^{λ·ψ} ψ - W, ψ = (1, ξ, |ξ|²/2), with the stall test and the
//     Armijo backtracking on Φ(λ) = Σ ω f e^{λ·ψ} - λ·W.  Every sum is a block reduction
//     (compensated in the mixed form); thread 0 takes the decisions and solves the symmetric
//     (dim+2)² Newton system in FP64 (Gaussian elimination, partial pivoting);
//  2. f₁ *= e^{λ·ψ}; f = f τ/(τ+Δt) + Δt/(τ+Δt) g⁺, g⁺ = M(prim_c)(1 + Shakhov(q)) (:181-185).
template <int D, typename A>
__device__ __forceinline__ void cip_psi(const A* VU, int64_t PG, int64_t goff, int i, A* ps) {
    ps[0] = (A)1;
    A s = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const A x = VU[(int64_t)d * PG + goff + i];
        ps[1 + d] = x;
        s += x * x;
    }
    ps[D + 1] = s / (A)2;
}
template <int M, typename A>
__device__ __forceinline__ A cip_dot(const A* lam, const A* ps) {
    A d = 0;
#pragma unroll
    for (int m = 0; m < M; ++m) d += lam[m] * ps[m];
    return d;
}
__device__ __forceinline__ double cip_exp(double x) { return exp(x); }
__device__ __forceinline__ float cip_exp(float x) { return expf(x); }

// conserved_I_porjection!'s solve for the cell of record FC (one CTA; every thread of the
// block takes part): f (the cell's block, in the storage type) has its negative values of f₁
// shaved in place; lam receives the multipliers λ in every thread.  w: the cell's conserved
// variables (FP64, padded to MAXW).
template <int D, int NDF, typename T>
__device__ __forceinline__ void iprojection_solve(const Dev& P, const FluxCell& FC, T* f, const double* wc,
                                                  double (&lamd)[D + 2]) {
    using A = typename Arith<T>::type;
    constexpr int M = D + 2, NJ = M * (M + 1) / 2, NS = M + NJ, MAXIT = 10;
    __shared__ double sred[NS * (BLOCK / 32)];
    __shared__ double slam[M], strial[M];
    __shared__ A slA[M];
    __shared__ int sctl;
    const int nv = FC.nv;
    const int64_t PG = P.PG, goff = FC.goff;
    const A* VU = vel<A>(P);
    const A* VW = wts<A>(P) + goff;

    // ---- W, and the shave of negative values of f₁ (I-projection.jl:78-88) ----------------
    {
        KSum<A> ei[1];
        double mn[2] = {-INFINITY, -INFINITY};   // -min f₁, -min of the positive f₁
        for (int i = threadIdx.x; i < nv; i += BLOCK) {
            const double x = (double)f[i];
            mn[0] = fmax(mn[0], -x);
            if (x > 0.0) mn[1] = fmax(mn[1], -x);
            if (NDF == 2) ei[0].add(VW[i] * (A)f[nv + i]);
        }
        double e[1];
        block_sum_ks<1, BLOCK>(ei, e, sred);
        block_max<2>(mn, sred);
        const double f_min = 1.1 * -mn[0], fp_min = -mn[1];
        if (f_min < 0.0 && fp_min < INFINITY) {
            const double dd = fp_min - f_min;
            for (int i = threadIdx.x; i < nv; i += BLOCK) {
                const double x = (double)f[i];
                if (x < 0.0) f[i] = (T)((x - f_min) / dd * fp_min);
            }
        }
        if (threadIdx.x == 0) {
            for (int m = 0; m < M; ++m) { slam[m] = 0.0; strial[m] = wc[m]; }
            if (NDF == 2) strial[M - 1] -= e[0] / 2;
        }
        __syncthreads();
    }
    // ---- Newton iterations (thread 0 keeps the state; the block evaluates the sums) ----------
    double W[M], dl[M], gprev = INFINITY, tol = 0.0, phi0 = 0.0, slope = 0.0, alpha = 1.0;
    int stall = 0;
#pragma unroll
    for (int m = 0; m < M; ++m) W[m] = strial[m];
    {
        double wn = 0.0;
#pragma unroll
        for (int m = 0; m < M; ++m) wn += W[m] * W[m];
        tol = 1e-10 * fmax(1.0, sqrt(wn));
    }
    for (int it = 0; it < MAXIT; ++it) {
        if (threadIdx.x < M) slA[threadIdx.x] = (A)slam[threadIdx.x];
        __syncthreads();
        A lam[M];
#pragma unroll
        for (int m = 0; m < M; ++m) lam[m] = slA[m];
        KSum<A> acc[NS];
        for (int i = threadIdx.x; i < nv; i += BLOCK) {
            A ps[M];
            cip_psi<D, A>(VU, PG, goff, i, ps);
            const A c = VW[i] * (A)f[i] * cip_exp(cip_dot<M, A>(lam, ps));
            int q = M;
#pragma unroll
            for (int a = 0; a < M; ++a) {
                const A ca = c * ps[a];
                acc[a].add(ca);
#pragma unroll
                for (int b = a; b < M; ++b) acc[q++].add(ca * ps[b]);
            }
        }
        double red[NS];
        block_sum_ks<NS, BLOCK>(acc, red, sred);
        if (threadIdx.x == 0) {
            double G[M], gn = 0.0;
#pragma unroll
            for (int m = 0; m < M; ++m) { G[m] = red[m] - W[m]; gn += G[m] * G[m]; }
            gn = sqrt(gn);
            int stop = 0;
            if (!(gn >= tol)) stop = 1;   // converged (or not a number)
            else if (gn > 0.9 * gprev) { if (++stall >= 2) stop = 1; }
            else stall = 0;
            if (!stop) {
                gprev = gn;
                double J[M][M], b[M];
                int q = M;
                for (int a = 0; a < M; ++a)
                    for (int c = a; c < M; ++c) { J[a][c] = red[q]; J[c][a] = red[q]; ++q; }
                for (int a = 0; a < M; ++a) b[a] = -G[a];
                for (int c = 0; c < M; ++c) {
                    int p = c;
                    for (int r = c + 1; r < M; ++r)
                        if (fabs(J[r][c]) > fabs(J[p][c])) p = r;
                    if (p != c) {
                        for (int j = 0; j < M; ++j) { const double t = J[c][j]; J[c][j] = J[p][j]; J[p][j] = t; }
                        const double t = b[c]; b[c] = b[p]; b[p] = t;
                    }
                    for (int r = c + 1; r < M; ++r) {
                        const double l = J[r][c] / J[c][c];
                        for (int j = c; j < M; ++j) J[r][j] -= l * J[c][j];
                        b[r] -= l * b[c];
                    }
                }
                for (int r = M - 1; r >= 0; --r) {
                    double sacc = b[r];
                    for (int j = r + 1; j < M; ++j) sacc -= J[r][j] * dl[j];
                    dl[r] = sacc / J[r][r];
                }
                double lw = 0.0;
                slope = 0.0;
                for (int m = 0; m < M; ++m) { lw += slam[m] * W[m]; slope += G[m] * dl[m]; }
                phi0 = red[0] - lw;   // Σ ω f e^{λ·ψ} is G's first sum (ψ₀ = 1)
                alpha = 1.0;
                for (int m = 0; m < M; ++m) strial[m] = slam[m] + dl[m];
            }
            sctl = stop;
        }
        __syncthreads();
        if (sctl) break;
        for (int ls = 0; ls < MAXIT; ++ls) {
            // FP64: Φ at the trial point, as the reference evaluates it.  Mixed form: the
            // difference Φ(λ + αΔλ) - Φ(λ) = Σ ω f e^{λ·ψ} expm1(αΔλ·ψ) - αΔλ·W, the same test in
            // exact arithmetic; FP32 terms could not resolve Φ's decrease near convergence
            // (~|G|²), and the solve would stall at |G| ~ 1e-4 |W|
            if (threadIdx.x < M) slA[threadIdx.x] = (A)(sizeof(A) == 8 ? strial[threadIdx.x] : strial[threadIdx.x] - slam[threadIdx.x]);
            __syncthreads();
            A dlt[M];
#pragma unroll
            for (int m = 0; m < M; ++m) dlt[m] = slA[m];
            KSum<A> a1[1];
            for (int i = threadIdx.x; i < nv; i += BLOCK) {
                A ps[M];
                cip_psi<D, A>(VU, PG, goff, i, ps);
                if constexpr (sizeof(A) == 8) {
                    a1[0].add(VW[i] * (A)f[i] * cip_exp(cip_dot<M, A>(dlt, ps)));
                } else {
                    const A c = VW[i] * (A)f[i] * cip_exp(cip_dot<M, A>(lam, ps));
                    a1[0].add(c * expm1f(cip_dot<M, A>(dlt, ps)));
                }
            }
            double r1[1];
            block_sum_ks<1, BLOCK>(a1, r1, sred);
            if (threadIdx.x == 0) {
                double lw = 0.0;
                bool ok;
                if constexpr (sizeof(A) == 8) {
                    for (int m = 0; m < M; ++m) lw += strial[m] * W[m];
                    ok = r1[0] - lw <= phi0 + 1e-4 * alpha * slope;
                } else {
                    for (int m = 0; m < M; ++m) lw += (strial[m] - slam[m]) * W[m];
                    ok = r1[0] - lw <= 1e-4 * alpha * slope;
                }
                if (ok) {
                    sctl = 1;
                } else {
                    alpha *= 0.5;
                    for (int m = 0; m < M; ++m) strial[m] = slam[m] + alpha * dl[m];
                    sctl = 0;
                }
            }
            __syncthreads();
            if (sctl) break;
        }
        if (threadIdx.x == 0)
            for (int m = 0; m < M; ++m) slam[m] += alpha * dl[m];
        __syncthreads();
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < M; ++m) lamd[m] = slam[m];
    __syncthreads();
}

// (2D mixed form: three CTAs per SM, with 4 bytes of spills, instead of two)
template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK, (D == 2 && sizeof(T) == 4) ? 3 : 1) cip_kernel(Dev P) {
    using A = typename Arith<T>::type;
    constexpr int M = D + 2;
    extern __shared__ __align__(16) unsigned char sh_raw[];
    __shared__ A slA[M];
    enum { C_PREC = 0, C_BFC, C_R1, C_R2, C_SK, C_LC, C_UH, C_UL = C_UH + MAXD, C_QA = C_UL + MAXD, C_N = C_QA + MAXD };
    __shared__ A sc[C_N];
    __shared__ float sUl[MAXD], sUh[MAXD], slh, sll;
    const FluxCell FC = P.fcrec[blockIdx.x];
    const int cell = FC.cell, slot = FC.slot, nv = FC.nv;
    const ProbParams& PP = P.probs[slot];
    const int64_t PG = P.PG, goff = FC.goff;
    const A* VU = vel<A>(P);
    T* f = (T*)P.f_out + FC.foff;
    double slam[M];
    iprojection_solve<D, NDF, T>(P, FC, f, P.w + (int64_t)cell * MAXW, slam);
    // ---- collision constants of prim_c (the flux kernel's expressions) ----------------------
    A* Ec = (A*)sh_raw;
    const double* pc = P.prim + (int64_t)cell * MAXW;
    if (threadIdx.x == 0) {
        bool bad = false;
        for (int m = 0; m < M; ++m) {
            slA[m] = (A)slam[m];
            bad |= !isfinite(slam[m]);
        }
        if (bad) atomicOr(&P.status[slot], ST_NONFINITE);
        const double lc = pc[D + 1];
        for (int d = 0; d < D; ++d) {
            const double x = pc[1 + d];
            sUh[d] = (float)x;
            sUl[d] = (float)(x - (double)sUh[d]);
            sc[C_UH + d] = (A)(sizeof(A) == 4 ? (double)sUh[d] : x);
            sc[C_UL + d] = (A)(sizeof(A) == 4 ? (double)sUl[d] : 0.0);
            sc[C_QA + d] = (A)P.qf[(int64_t)cell * MAXD + d];
        }
        slh = (float)lc;
        sll = (float)(lc - (double)slh);
        if constexpr (sizeof(A) == 8) {
            const double tau = PP.mu_ref * 2.0 * pow(lc, 1.0 - PP.omega) / pc[0];
            sc[C_PREC] = pc[0] * (D == 2 ? lc / PI : pow(lc / PI, 1.5));
            sc[C_BFC] = PP.K / (2.0 * lc);
            sc[C_R1] = tau / (tau + PP.dt);
            sc[C_R2] = PP.dt / (tau + PP.dt);
            sc[C_SK] = 0.8 * (1.0 - PP.Pr) * lc * lc / pc[0];
            sc[C_LC] = lc;
        } else {
            const float rc = (float)pc[0], lcf = slh, dtf = PP.dtf;
            const float tau = PP.mu2f * powf(lcf, PP.omf) / rc;
            constexpr float IPI = (float)(1.0 / PI);
            sc[C_PREC] = rc * (D == 2 ? lcf * IPI : powf(lcf * IPI, 1.5f));
            sc[C_BFC] = PP.Kf / (2.f * lcf);
            sc[C_R1] = tau / (tau + dtf);
            sc[C_R2] = dtf / (tau + dtf);
            sc[C_SK] = PP.shkf * lcf * lcf / rc;
            sc[C_LC] = lcf;
        }
    }
    __syncthreads();
    if constexpr (sizeof(A) == 8) {
        double U[D];
        for (int d = 0; d < D; ++d) U[d] = pc[1 + d];
        gauss_table<D, BLOCK>(P, FC.gid, U, pc[D + 1], (double*)Ec);
    } else {
        gauss_table<D, BLOCK>(P, FC.gid, sUh, sUl, slh, sll, (float*)Ec);
    }
    __syncthreads();
    // ---- f₁ e^{λ·ψ}, then the relaxation towards g⁺ ----------------------------------------
    const int MA = P.max_axis;
    const uint16_t* vx = P.vidx + goff;
    const A prec = sc[C_PREC], bfc = sc[C_BFC], r1 = sc[C_R1], r2 = sc[C_R2], sk = sc[C_SK], lc = sc[C_LC];
    const A Kk = (A)PP.K;
    A lam[M], Uh[D], Ul[D], qa[D];
#pragma unroll
    for (int m = 0; m < M; ++m) lam[m] = slA[m];
#pragma unroll
    for (int d = 0; d < D; ++d) { Uh[d] = sc[C_UH + d]; Ul[d] = sc[C_UL + d]; qa[d] = sc[C_QA + d]; }
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        A ps[M];
        cip_psi<D, A>(VU, PG, goff, i, ps);
        A fv[NDF];
        fv[0] = (A)f[i] * cip_exp(cip_dot<M, A>(lam, ps));
        if (NDF == 2) fv[NDF - 1] = (A)f[nv + i];
        A mc = prec;
#pragma unroll
        for (int d = 0; d < D; ++d) mc *= Ec[d * MA + vx[(int64_t)d * PG + i]];
        A c2 = 0, cq = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const A cd = (VU[(int64_t)d * PG + goff + i] - Uh[d]) - Ul[d];
            c2 += cd * cd;
            cq += cd * qa[d];
        }
        A gp[NDF];
        if (NDF == 2) {
            const A mb = mc * bfc;
            gp[0] = mc + sk * cq * ((A)2 * lc * c2 + Kk - (A)5) * mc;
            gp[NDF - 1] = mb + sk * cq * ((A)2 * lc * c2 + Kk - (A)3) * mb;
        } else {
            gp[0] = mc + sk * cq * ((A)2 * lc * c2 - (A)5) * mc;
        }
#pragma unroll
        for (int k = 0; k < NDF; ++k) f[k * nv + i] = (T)(fv[k] * r1 + r2 * gp[k]);
    }
}

// vs_conserved_correction! (Velocity_space/AMR.jl:122-137): conserved_I_porjection! of the
// listed fluid-list entries on the current f (in place) and w, one CTA each.
template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK) conserve_kernel(Dev P, const int32_t* list) {
    using A = typename Arith<T>::type;
    constexpr int M = D + 2;
    const FluxCell FC = P.fcrec[list[blockIdx.x]];
    T* f = (T*)P.f_in + FC.foff;
    double lam[M];
    iprojection_solve<D, NDF, T>(P, FC, f, P.w + (int64_t)FC.cell * MAXW, lam);
    A la[M];
    bool bad = false;
#pragma unroll
    for (int m = 0; m < M; ++m) { la[m] = (A)lam[m]; bad |= !isfinite(lam[m]); }
    if (bad && threadIdx.x == 0) atomicOr(&P.status[FC.slot], ST_NONFINITE);
    const A* VU = vel<A>(P);
    for (int i = threadIdx.x; i < FC.nv; i += BLOCK) {
        A ps[M];
        cip_psi<D, A>(VU, P.PG, FC.goff, i, ps);
        f[i] = (T)((A)f[i] * cip_exp(cip_dot<M, A>(la, ps)));
    }
}

// save_boundary_result! (Boundary/Immersed_boundary.jl:12-61) from the wall distribution the
// wall kernel just rebuilt in each SolidNeighbor record's f block (the donor's velocity grid):
// aux_w = calc_w0, aux_prim = get_prim(aux_w), aux_qf = calc_qf(aux_prim) and the pressure
// tensor Σ w u_a u_b h (pressure_2D / pressure_3D, lib/KitCore/2D.jl:31-37, 3D.jl:37-46), all
// in FP64.  One CTA per record; out row: prim (D+2), qf (D), p (D (D+1) / 2).
template <int D, int NDF, typename T>
__global__ void __launch_bounds__(BLOCK) wall_rows_kernel(Dev P, double* out) {
    constexpr int NP = D * (D + 1) / 2;
    constexpr int N1 = D + 2 + NP;
    constexpr int W = D + 2 + D + NP;
    __shared__ double sred[N1 * (BLOCK / 32)];
    __shared__ double sprim[MAXW];
    const WallOp op = P.wall_ops[blockIdx.x];
    const VGridView g = grid_view(P, op.donor);
    const int nv = g.nv;
    const T* wf = (const T*)P.f_in + P.foff[op.data];
    double v[N1];
#pragma unroll
    for (int q = 0; q < N1; ++q) v[q] = 0.0;
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        const double wt = P.vw[g.goff + i];
        const double h = (double)wf[i];
        const double b = NDF == 2 ? (double)wf[(NDF - 1) * nv + i] : 0.0;
        double u[D], u2 = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) { u[d] = g.u(i, d); u2 += u[d] * u[d]; }
        v[0] += wt * h;
#pragma unroll
        for (int d = 0; d < D; ++d) v[1 + d] += wt * u[d] * h;
        v[D + 1] += NDF == 2 ? 0.5 * wt * (u2 * h + b) : 0.5 * wt * u2 * h;
        int e = D + 2;
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int c = a; c < D; ++c) v[e++] += u[a] * u[c] * h * wt;
    }
    block_sum<N1>(v, sred);
    if (threadIdx.x == 0) get_prim<D>(v, P.probs[P.dprob[op.donor]].gamma, sprim);
    __syncthreads();
    double q[D];
#pragma unroll
    for (int d = 0; d < D; ++d) q[d] = 0.0;
    for (int i = threadIdx.x; i < nv; i += BLOCK) {
        const double wt = P.vw[g.goff + i];
        const double h = (double)wf[i];
        const double b = NDF == 2 ? (double)wf[(NDF - 1) * nv + i] : 0.0;
        double c[D], c2 = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) { c[d] = g.u(i, d) - sprim[1 + d]; c2 += c[d] * c[d]; }
        const double hb = NDF == 2 ? c2 * h + b : c2 * h;
#pragma unroll
        for (int d = 0; d < D; ++d) q[d] += 0.5 * wt * c[d] * hb;
    }
    block_sum<D>(q, sred);
    if (threadIdx.x == 0) {
        double* o = out + (int64_t)blockIdx.x * W;
        for (int e = 0; e < D + 2; ++e) o[e] = sprim[e];
        for (int d = 0; d < D; ++d) o[D + 2 + d] = q[d];
        for (int e = 0; e < NP; ++e) o[2 * D + 2 + e] = v[D + 2 + e];
    }
}

// an ordinary launch, or one with programmatic stream serialization (pdl: a programmatic
// dependent of the kernel before it on the stream)
template <typename... Args>
static cudaError_t launch_pdl(void (*fn)(Args...), int grid, int nt, size_t smem, cudaStream_t s, bool pdl, Args... args) {
    if (!pdl) {
        fn<<<grid, nt, smem, s>>>(args...);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)nt);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, fn, args...);
}

template <int D, int NDF, typename T>
struct Launch {
    // the slope work items [item_base, item_base + n) of one pass
    static cudaError_t slope(const Dev& P, int item_base, int n, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        if (P.slope_nt == 128) slope_kernel<D, NDF, T, 128><<<n, 128, 0, s>>>(P, item_base);
        else slope_kernel<D, NDF, T, BLOCK><<<n, BLOCK, 0, s>>>(P, item_base);
        return cudaGetLastError();
    }
    static cudaError_t solid(const Dev& P, int n, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        solid_kernel<D, NDF, T><<<n, BLOCK, 0, s>>>(P);
        return cudaGetLastError();
    }
    static cudaError_t wall_rows(const Dev& P, int n, double* out, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        wall_rows_kernel<D, NDF, T><<<n, BLOCK, 0, s>>>(P, out);
        return cudaGetLastError();
    }
    static cudaError_t wall(const Dev& P, int n, int max_nv, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        size_t smem = wall_smem<D, NDF, typename Arith<T>::type>(max_nv, P.max_axis);
        cudaError_t e = cudaFuncSetAttribute(wall_kernel<D, NDF, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        wall_kernel<D, NDF, T><<<n, BLOCK, smem, s>>>(P);
        return cudaGetLastError();
    }
    // the flux kernel of the layout's staging choice
    using FluxFn = void (*)(Dev, int*, const int32_t*, int);
    // (list: one CTA per cell, schedule 0; the 2D mixed form's variant then takes 80 registers
    // and 6 resident 128-thread CTAs: beside the packed kernels on the other stream it shortened
    // the cylinder's step 1.52 -> 1.47 ms, while the persistent schedule of a batch, whose
    // autotuned grid counts on 8 resident CTAs, keeps 64; the same arithmetic either way)
    static FluxFn flux_fn(const Dev& P, bool list = false) {
        // CIP marching on a layout with walls: the variant with positivity_preserving_ib!
        if (P.marching == KG_MARCH_CIP && P.n_walls > 0)
            return P.fst_global ? flux_collide_kernel<D, NDF, T, true, BLOCK, true> : flux_collide_kernel<D, NDF, T, false, BLOCK, true>;
        if (P.fst_global) return flux_collide_kernel<D, NDF, T, true, BLOCK>;
        if (D == 2 && sizeof(T) == 4 && list && P.flux_nt == 128) return flux_collide_kernel<D, NDF, T, false, 128, false, 3>;
        return P.flux_nt == 128 ? flux_collide_kernel<D, NDF, T, false, 128> : flux_collide_kernel<D, NDF, T, false, BLOCK>;
    }
    static int flux_threads(const Dev& P) {
        return (P.fst_global || (P.marching == KG_MARCH_CIP && P.n_walls > 0)) ? BLOCK : (P.flux_nt == 128 ? 128 : BLOCK);
    }
    // one CTA per listed fluid-list entry
    static cudaError_t flux_list(const Dev& P, const int32_t* list, int n, int max_nv, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        using A = typename Arith<T>::type;
        size_t smem = flux_smem<D, NDF, A>(max_nv, P.max_axis, P.max_bcm, P.fst_global);
        const FluxFn fn = flux_fn(P, true);
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        fn<<<n, flux_threads(P), smem, s>>>(P, nullptr, list, n);
        return cudaGetLastError();
    }
    // the regular-cell kernel, one CTA per listed fluid-list entry (every one regular)
    // (pdl: the packed kernel launched as a programmatic dependent of the packed-form kernel
    // before it)
    static cudaError_t flux_reg_list(const Dev& P, const int32_t* list, int n, int max_nv, cudaStream_t s,
                                     bool pdl = false) {
        if (n <= 0) return cudaSuccess;
        using A = typename Arith<T>::type;
        size_t smem = flux_smem<D, NDF, A>(max_nv, P.max_axis, P.max_bcm, P.fst_global);
        using RegFn = void (*)(Dev, const int32_t*);
        // (the CTA size of the layout; the generic kernel's CIP variant for layouts with walls
        // runs 256 threads, which does not concern regular cells)
        const int nt = P.fst_global ? BLOCK : (P.flux_nt == 128 ? 128 : BLOCK);
        RegFn fn = P.fst_global ? flux_regular_kernel<D, NDF, T, true, BLOCK>
                                : (P.flux_nt == 128 ? flux_regular_kernel<D, NDF, T, false, 128>
                                                    : flux_regular_kernel<D, NDF, T, false, BLOCK>);
        int ntl = nt;
        if constexpr (D == 2 && NDF == 2 && sizeof(T) == 4) {
            // the packed-FP32 kernel (its convected f always in shared memory; 64 threads for
            // layouts of small velocity grids)
            if (!P.fst_global && P.marching != KG_MARCH_CIP) {
                fn = P.packed_nt == 64 ? flux_packed_kernel<64, PACKED_VPT, false>
                   : (P.flux_nt == 128 ? flux_packed_kernel<128, PACKED_VPT, false> : flux_packed_kernel<BLOCK, PACKED_VPT, false>);
                ntl = P.packed_nt == 64 ? 64 : nt;
                smem = packed_smem(max_nv, P.max_axis);
            }
        }
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        return launch_pdl(fn, n, ntl, smem, s, pdl, P, list);
    }
    // the packed kernel of the R2 cells (slopes from f), one CTA per listed entry
    static cudaError_t flux_r2_list(const Dev& P, const int32_t* list, int n, int max_nv, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        if constexpr (D == 2 && NDF == 2 && sizeof(T) == 4) {
            using A = typename Arith<T>::type;
            const size_t smem = packed_smem(max_nv, P.max_axis);
            const int nt = P.packed_nt == 64 ? 64 : (P.flux_nt == 128 ? 128 : BLOCK);
            using RegFn = void (*)(Dev, const int32_t*);
            RegFn fn = nt == 64 ? flux_packed_kernel<64, R2_VPT, true>
                     : (nt == 128 ? flux_packed_kernel<128, R2_VPT, true> : flux_packed_kernel<BLOCK, R2_VPT, true>);
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            fn<<<n, nt, smem, s>>>(P, list);
            return cudaGetLastError();
        }
        return cudaErrorInvalidValue;   // R2 lists exist only for the 2D mixed form
    }
    // the packed kernel's INNER form, one CTA per listed entry (2D mixed form)
    // (pdl: launched as a programmatic dependent of the packed-form kernel before it)
    static cudaError_t flux_inner_list(const Dev& P, const int32_t* list, int n, int max_nv, bool paired, cudaStream_t s,
                                       bool pdl) {
        if (n <= 0) return cudaSuccess;
        if constexpr (D == 2 && NDF == 2 && sizeof(T) == 4) {
            const size_t smem = packed_smem(max_nv, P.max_axis);
            using RegFn = void (*)(Dev, const int32_t*);
            const int nt = P.packed_nt == 64 ? 64 : (P.flux_nt == 128 ? 128 : BLOCK);
            RegFn fn = paired ? (nt == 64 ? flux_packed_inner_kernel<64, true>
                               : (nt == 128 ? flux_packed_inner_kernel<128, true> : flux_packed_inner_kernel<BLOCK, true>))
                              : (nt == 64 ? flux_packed_inner_kernel<64, false>
                               : (nt == 128 ? flux_packed_inner_kernel<128, false> : flux_packed_inner_kernel<BLOCK, false>));
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            return launch_pdl(fn, n, nt, smem, s, pdl, P, list);
        }
        return cudaErrorInvalidValue;   // inner lists exist only for the 2D mixed form
    }
    // persistent schedule: `grid` resident CTAs; the counter must be zero at launch
    static cudaError_t flux_persistent(const Dev& P, int n, int max_nv, int grid, int* counter, const int32_t* order,
                                       cudaStream_t s) {
        using A = typename Arith<T>::type;
        size_t smem = flux_smem<D, NDF, A>(max_nv, P.max_axis, P.max_bcm, P.fst_global);
        const FluxFn fn = flux_fn(P);
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaMemsetAsync(counter, 0, sizeof(int), s);
        if (e != cudaSuccess) return e;
        fn<<<grid, flux_threads(P), smem, s>>>(P, counter, order, n);
        return cudaGetLastError();
    }
    // CIP_Marching's I-projection and relaxation of the fluid cells (after the flux kernel)
    static cudaError_t cip(const Dev& P, int n, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        using A = typename Arith<T>::type;
        const size_t smem = (size_t)D * P.max_axis * sizeof(A);
        cudaError_t e = cudaFuncSetAttribute(cip_kernel<D, NDF, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        cip_kernel<D, NDF, T><<<n, BLOCK, smem, s>>>(P);
        return cudaGetLastError();
    }
    // vs_conserved_correction! of n listed fluid-list entries
    static cudaError_t conserve(const Dev& P, const int32_t* list, int n, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        conserve_kernel<D, NDF, T><<<n, BLOCK, 0, s>>>(P, list);
        return cudaGetLastError();
    }
    static cudaError_t macro_slope(const Dev& P, int fbegin, int n, int dbase, double* out, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        macro_slope_kernel<D, NDF, T><<<n, BLOCK, 0, s>>>(P, fbegin, dbase, out);
        return cudaGetLastError();
    }
    // velocity-space adaptation: resolution terms, then flags, of the cells [c0, c0 + n)
    static cudaError_t vs_resolution(const Dev& P, int c0, int n, double* out, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        vs_resolution_kernel<D, NDF, T><<<n, BLOCK, 0, s>>>(P, c0, out);
        return cudaGetLastError();
    }
    static cudaError_t vs_flags(const Dev& P, int c0, int n, const VsFlagArgs& A, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        vs_flags_kernel<D, NDF, T><<<n, BLOCK, 0, s>>>(P, c0, A);
        return cudaGetLastError();
    }
    // adapted-mesh state from the previous pools, one CTA per cell record
    static cudaError_t adapt(const Dev& P, int n, const AdaptRec* recs, const void* f, const void* sdf, const double* w,
                             const double* prim, const double* qf, const int32_t* runs, const int8_t* lev,
                             cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        AdaptView<T> V{recs, (const T*)f, (const T*)sdf, w, prim, qf, runs, lev};
        adapt_kernel<D, NDF, T><<<n, BLOCK, 0, s>>>(P, V);
        return cudaGetLastError();
    }
    // physical-space criterion of the fluid cells [fbegin, fbegin + n): loh from sw, then
    // the buffer layer into out (both per data item from dbase on)
    static cudaError_t criterion(const Dev& P, int fbegin, int n, int dbase, const double* sw, double thr,
                                 double* loh, double* out, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        const int nb = (n + 127) / 128;
        criterion_kernel<D><<<nb, 128, 0, s>>>(P, fbegin, n, dbase, sw, loh);
        criterion_buffer_kernel<D><<<nb, 128, 0, s>>>(P, fbegin, n, dbase, thr, loh, out);
        return cudaGetLastError();
    }
    // resident CTAs per SM the flux kernel reaches (for the persistent grid size)
    static int flux_occupancy(const Dev& P, int max_nv) {
        using A = typename Arith<T>::type;
        size_t smem = flux_smem<D, NDF, A>(max_nv, P.max_axis, P.max_bcm, P.fst_global);
        const FluxFn fn = flux_fn(P);
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, flux_threads(P), smem);
        return nb;
    }
};

cudaError_t launch_residual(const Dev& P, const int32_t* live, int n_live, double* out, cudaStream_t s) {
    if (n_live <= 0) return cudaSuccess;
    residual_kernel<<<n_live, BLOCK, 0, s>>>(P, live, out);
    return cudaGetLastError();
}

// explicit instantiations: 2D two-distribution and 3D one-distribution, plain and mixed
template struct Launch<2, 2, double>;
template struct Launch<3, 1, double>;
template struct Launch<2, 2, float>;
template struct Launch<3, 1, float>;

}  // namespace kg
