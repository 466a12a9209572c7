// kg_devflat.cu -- the gather form of one problem built on the device.
//
// amr_recover! (Solver/AMR.jl:54-70) rebuilds the faces and neighbours of the adapted forest
// (initialize_faces!, Solver/Initialize.jl:5-158).  Here the records a step reads are rebuilt
// from those reference-shaped arrays by kernels, one thread per cell or per face: the slope
// operations of slope! and their neighbour lists, the dependency depth of the slope passes,
// the criterion rows, the per-cell face incidences (the gather form of flux!) with the
// regular-cell test, and the per-cell flux and slope records.  The host keeps what is small
// or serial: the argument checks, the velocity grids and their pairing tables, the data table
// and the immersed-boundary records.  Every array equals the host builder's (kg_flatten.cpp)
// byte for byte; the kernels restate its decisions in the same order, and this file is
// compiled without FMA contraction so every double expression rounds as the host's does.
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cstring>
#include "kg_device.cuh"
#include "kg_devflat.h"

namespace kg {
namespace {

enum DfErr {
    DF_OK = 0, DF_BOTH_BOUNDARY = 1, DF_BAD_STATE = 2, DF_LIST_NOTHING = 3, DF_LIST_LONG = 4, DF_PAIR = 5
};

// device view of the topology and the host-built tables
struct DT {
    int D, NC, NWL, NFACE, G, half, lmin;
    const int32_t *be, *lev, *grid;
    const double *mid, *ds;
    const int8_t* nst;
    const int32_t *noff, *nref;
    const int8_t *fkind, *fdir;
    const double *frot, *farea, *fmid;
    const int32_t *fhere, *fthere;
    const double* ftmid;
    const int8_t* fbck;
    const double *fbc, *waux;
    const int64_t *foff, *g_off;
    const int32_t *dgrid, *dbe, *dnv;
    const double *dmid, *dds, *dinvv;
    const int32_t* pair;      // G x G pairing ids (-1: none)
    int* err;                 // [code, item]
};

__device__ __forceinline__ void df_fail(const DT& T, int code, int item) {
    if (atomicCAS(T.err, 0, code) == 0) T.err[1] = item;
}
__device__ __forceinline__ int d_data_of(const DT& T, int32_t r) {
    if (r == KG_NBR_NONE || r == KG_NBR_INSIDE) return -1;
    if (r >= 0) return r;
    return T.NC + (-1 - r);
}
__device__ __forceinline__ int d_pair(const DT& T, int ga, int gb, int item, bool* ok) {
    if (ga == gb) return -1;
    const int p = T.pair[(size_t)ga * T.G + gb];
    if (p < 0) { df_fail(T, DF_PAIR, item); *ok = false; }
    return p;
}

// ---- slope! operations of one pass-cell entry (the host builder's dispatch / transverse) ----
// FILL: write the D ops at ops[k * D] and the neighbour entries from nbr[base]; returns the
// number of neighbour entries, or -1 after an error
template <bool FILL>
__device__ int slope_entry(const DT& T, int k, int cell, SlopeOp* ops, NbrRef* nbr, int base) {
    const int D = T.D, NF = 2 * D;
    int used = 0;
    bool ok = true;
    auto st = [&](int kk) { return (int)T.nst[cell * NF + kk]; };
    auto cnt = [&](int kk) { return (int)(T.noff[cell * NF + kk + 1] - T.noff[cell * NF + kk]); };
    auto lst = [&](int kk) { return T.nref + T.noff[cell * NF + kk]; };
    auto first_data = [&](int kk) { return d_data_of(T, lst(kk)[0]); };
    auto be_of = [&](int dn) -> int {
        if (dn < 0) { df_fail(T, DF_LIST_NOTHING, cell); ok = false; return 0; }
        return T.dbe[dn];
    };
    auto dmid_of = [&](int dn, int d) -> double { return dn < 0 ? 0.0 : T.dmid[(size_t)dn * MAXD + d]; };
    auto add_list = [&](int kk, int32_t& off, int32_t& n) {
        off = base + used;
        n = cnt(kk);
        const int32_t* l = lst(kk);
        for (int j = 0; j < n; ++j) {
            const int dn = d_data_of(T, l[j]);
            if (dn < 0) { df_fail(T, DF_LIST_NOTHING, cell); ok = false; return; }
            const int p = d_pair(T, T.grid[cell], T.dgrid[dn], cell, &ok);
            if (FILL) nbr[off + j] = NbrRef{dn, p};
        }
        used += n;
    };
    auto has_offset = [&](int kk) {   // _ps_has_transverse_offset (Slope.jl:177-199)
        const int dir = kk / 2, n = cnt(kk);
        if (n == 0) return false;
        for (int tt = 0; tt < D; ++tt) {
            if (tt == dir) continue;
            double avg = 0.0;
            for (int j = 0; j < n; ++j) avg += dmid_of(d_data_of(T, lst(kk)[j]), tt);
            avg /= n;
            if (avg != T.mid[(size_t)cell * D + tt]) return true;
        }
        return false;
    };
    auto op_one = [&](SlopeOp& op, int kk, double dsv, bool proj) {
        op.kind = SLOPE_ONE; op.inv_dsA = 1.0 / dsv; op.projA = proj;
        add_list(kk, op.listA, op.cntA);
    };
    auto op_two = [&](SlopeOp& op, double dsL, double dsR, bool pL, bool pR, int dir) {
        op.kind = SLOPE_TWO; op.inv_dsA = 1.0 / dsL; op.inv_dsB = 1.0 / dsR; op.projA = pL; op.projB = pR;
        add_list(2 * dir, op.listA, op.cntA);
        if (ok) add_list(2 * dir + 1, op.listB, op.cntB);
    };
    const int L = T.lev[cell];
    const double* pm = T.mid + (size_t)cell * D;
    for (int dir = 0; dir < D && ok; ++dir) {
        SlopeOp op;
        op.inv_dsA = 0.0; op.inv_dsB = 0.0;
        op.listA = 0; op.cntA = 0; op.listB = 0; op.cntB = 0;
        op.kind = SLOPE_SKIP; op.projA = 0; op.projB = 0; op.dir = (int8_t)dir;
        op.cell = cell;
        const int kL = 2 * dir, kR = 2 * dir + 1;
        const int sL = st(kL), sR = st(kR);
        if (L == T.lmin || !(sL == -1 || sR == -1)) {
            // update_slope!(Val(sL), Val(sR)) (Slope.jl:458-771)
            const double dsv = T.ds[(size_t)cell * D + dir];
            if (sL == 1 && sR == 1) {
                const bool Ls = be_of(first_data(kL)) < 0, Rs = be_of(first_data(kR)) < 0;
                if (!ok) break;
                if (Ls && Rs) op.kind = SLOPE_ZERO;
                else if (Ls) op_one(op, kR, pm[dir] - dmid_of(first_data(kR), dir), false);
                else if (Rs) op_one(op, kL, pm[dir] - dmid_of(first_data(kL), dir), false);
                else op_two(op, dsv, -dsv, false, false, dir);
            } else if (sL == 0 || sR == 0) {
                if (sL == 0 && sR == 0) { df_fail(T, DF_BOTH_BOUNDARY, cell); ok = false; break; }
                const int kk = sL == 0 ? kR : kL;
                op_one(op, kk, pm[dir] - dmid_of(first_data(kk), dir), false);
            } else {
                const int half = T.half;
                if ((sL != 1 && sL != half && sL != -1) || (sR != 1 && sR != half && sR != -1)) {
                    df_fail(T, DF_BAD_STATE, cell); ok = false; break;
                }
                auto fac = [&](int s) { return s == 1 ? 1.0 : (s == half ? 0.75 : 1.5); };
                op_two(op, fac(sL) * dsv, -fac(sR) * dsv, false, false, dir);
            }
        } else {
            // transverse correction (update_slope_transverse_level!, Slope.jl:908-941)
            if (sL != 0 && sR != 0) {
                const int dL = first_data(kL), dR = first_data(kR);
                const double dsL = pm[dir] - dmid_of(dL, dir);
                const double dsR = pm[dir] - dmid_of(dR, dir);
                const bool Ls = be_of(dL) < 0;
                if (!ok) break;
                if (Ls) op_one(op, kR, dsR, true);
                else {
                    const bool Rs = be_of(dR) < 0;
                    if (!ok) break;
                    if (Rs) op_one(op, kL, dsL, true);
                    else op_two(op, dsL, dsR, has_offset(kL), has_offset(kR), dir);
                }
            } else if (sR == 0 && sL == -1) {
                const int dL = first_data(kL);
                const bool Ls = be_of(dL) < 0;
                if (!ok) break;
                if (Ls) op.kind = SLOPE_SKIP;
                else op_one(op, kL, pm[dir] - dmid_of(dL, dir), true);
            } else if (sL == 0 && sR == -1) {
                const int dR = first_data(kR);
                const bool Rs = be_of(dR) < 0;
                if (!ok) break;
                if (Rs) op.kind = SLOPE_SKIP;
                else op_one(op, kR, pm[dir] - dmid_of(dR, dir), true);
            } else {
                op.kind = SLOPE_SKIP;
            }
        }
        if (FILL && ok) ops[(size_t)k * D + dir] = op;
    }
    if (!ok) return -1;
    if (used > 2 * MAXD * 4) { df_fail(T, DF_LIST_LONG, cell); return -1; }
    return used;
}

__global__ void k_slope_count(DT T, const int32_t* pcells, int npc, int32_t* cnt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npc) return;
    const int n = slope_entry<false>(T, k, pcells[k], nullptr, nullptr, 0);
    cnt[k] = n < 0 ? 0 : n;
}
__global__ void k_slope_fill(DT T, const int32_t* pcells, int npc, const int32_t* base, SlopeOp* ops, NbrRef* nbr,
                             int32_t* cell_op) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npc) return;
    slope_entry<true>(T, k, pcells[k], ops, nbr, base[k]);
    cell_op[k] = k * T.D;
}

// One sweep of the dependency depth of the slope passes: an entry's depth is one more than the
// deepest coarser entry whose slope its transverse projection reads (longest path in the DAG of
// those reads, by repeated sweeps); flags[0]: a depth changed, flags[1]: a read of an entry not
// earlier in the level order (the layout keeps one pass per level).
__global__ void k_depth(DT T, const SlopeOp* ops, const NbrRef* nbr, const int32_t* entry, int npc, const int32_t* din,
                        int32_t* dout, int* flags) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npc) return;
    int dk = 0;
    for (int dir = 0; dir < T.D; ++dir) {
        const SlopeOp op = ops[(size_t)k * T.D + dir];
        if (op.kind != SLOPE_ONE && op.kind != SLOPE_TWO) continue;
        for (int side = 0; side < 2; ++side) {
            const bool proj = side == 0 ? op.projA : (op.kind == SLOPE_TWO && op.projB);
            if (!proj) continue;
            const int32_t l0 = side == 0 ? op.listA : op.listB, n = side == 0 ? op.cntA : op.cntB;
            for (int32_t j = 0; j < n; ++j) {
                const int32_t dn = nbr[l0 + j].data;
                if (dn >= T.NC || entry[dn] < 0) continue;
                if (entry[dn] >= k) { flags[1] = 1; continue; }
                dk = max(dk, din[entry[dn]] + 1);
            }
        }
    }
    dout[k] = dk;
    if (dk != din[k]) flags[0] = 1;
}

// Stable partition of the entries by depth (one CTA): the entries of depth 0 in level order,
// then depth 1, ...; offs[d] = first position of depth d, offs[maxd + 1] = npc.
__global__ void __launch_bounds__(1024) k_partition(const int32_t* depth, int npc, int maxd, const int32_t* pc_in,
                                                    int32_t* pc_out, int32_t* op_out, int32_t* offs, int D) {
    __shared__ int32_t ws[32];
    __shared__ int32_t tot;
    int pos = 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int d = 0; d <= maxd; ++d) {
        if (threadIdx.x == 0) offs[d] = pos;
        for (int c0 = 0; c0 < npc; c0 += 1024) {
            const int k = c0 + threadIdx.x;
            const int fl = (k < npc && depth[k] == d) ? 1 : 0;
            int x = fl;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) ws[wid] = x;
            __syncthreads();
            if (wid == 0) {
                int v = ws[lane];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, v, o);
                    if (lane >= o) v += y;
                }
                ws[lane] = v;
                if (lane == 31) tot = v;
            }
            __syncthreads();
            const int excl = x - fl + (wid > 0 ? ws[wid - 1] : 0);
            if (fl) {
                pc_out[pos + excl] = pc_in[k];
                op_out[pos + excl] = k * D;
            }
            pos += tot;
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) offs[maxd + 1] = pos;
}

// Exclusive prefix sum of n int32 counts into out[0..n] (one CTA).
__global__ void __launch_bounds__(1024) k_scan(const int32_t* in, int n, int32_t* out) {
    __shared__ int32_t ws[32];
    __shared__ int32_t carry;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < n; c0 += 1024) {
        const int k = c0 + threadIdx.x;
        const int v = k < n ? in[k] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int s = ws[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            ws[lane] = s;
        }
        __syncthreads();
        const int excl = carry + x - v + (wid > 0 ? ws[wid - 1] : 0);
        if (k < n) out[k] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

// ---- update_criterion! rows (per fluid cell and direction) -----------------------------------
__device__ __forceinline__ int crit_count(const DT& T, int cell) {
    const int D = T.D, NF = 2 * D;
    int n = 0;
    for (int k = 0; k < NF; ++k)
        if (T.nst[cell * NF + k] != 0) n += T.noff[cell * NF + k + 1] - T.noff[cell * NF + k];
    return n;
}
__global__ void k_crit_count(DT T, const int32_t* fluid, int nfl, int32_t* cnt) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nfl) cnt[q] = crit_count(T, fluid[q]);
}
__global__ void k_crit_fill(DT T, const int32_t* fluid, int nfl, const int32_t* base, CritOp* ops, int32_t* nbr) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nfl) return;
    const int i = fluid[q], D = T.D, NF = 2 * D;
    int at = base[q];
    for (int dir = 0; dir < D; ++dir) {
        CritOp op;
        op.listA = 0; op.cntA = 0; op.listB = 0; op.cntB = 0; op.pad = 0; op.pad2 = 0;
        const int sA = T.nst[i * NF + 2 * dir], sB = T.nst[i * NF + 2 * dir + 1];
        const double dsv = T.ds[(size_t)i * D + dir];
        auto factor = [](int s) { return s == 1 ? 1.0 : (s == -1 ? 1.5 : 0.75); };
        auto add = [&](int k, int32_t& l0, int32_t& n) {
            l0 = at;
            n = T.noff[i * NF + k + 1] - T.noff[i * NF + k];
            const int32_t* l = T.nref + T.noff[i * NF + k];
            for (int j = 0; j < n; ++j) nbr[at + j] = l[j] >= 0 ? l[j] : -1;
            at += n;
        };
        if (sA != 0) add(2 * dir, op.listA, op.cntA);
        if (sB != 0) add(2 * dir + 1, op.listB, op.cntB);
        op.dsA = factor(sA) * dsv;
        op.dsB = factor(sB) * dsv;
        op.coarseA = sA == -1;
        op.coarseB = sB == -1;
        op.kind = (sA != 0 && sB != 0) ? 1 : 0;
        ops[(size_t)q * D + dir] = op;
    }
}

// ---- flux incidences (flux!, Flux/Flux.jl:19-111,458-503) in the gather form -----------------
__global__ void k_inc_count(DT T, int32_t* nper, int32_t* isdom) {
    const int fi = blockIdx.x * blockDim.x + threadIdx.x;
    if (fi >= T.NFACE) return;
    atomicAdd(&nper[T.fhere[fi]], 1);
    const bool dom = T.fkind[fi] == KG_FACE_DOMAIN;
    isdom[fi] = dom ? 1 : 0;
    if (!dom) {
        const int od = d_data_of(T, T.fthere[fi]);
        if (od >= 0 && od < T.NC && T.dbe[od] >= 0) atomicAdd(&nper[od], 1);
    }
}
// each face's entries into its cells' runs (in any order; sorted by face per cell later)
__global__ void k_inc_place(DT T, const int32_t* pref, int32_t* fillc, int32_t* keys) {
    const int fi = blockIdx.x * blockDim.x + threadIdx.x;
    if (fi >= T.NFACE) return;
    const int here = T.fhere[fi];
    keys[pref[here] + atomicAdd(&fillc[here], 1)] = 2 * fi;
    if (T.fkind[fi] != KG_FACE_DOMAIN) {
        const int od = d_data_of(T, T.fthere[fi]);
        if (od >= 0 && od < T.NC && T.dbe[od] >= 0) keys[pref[od] + atomicAdd(&fillc[od], 1)] = 2 * fi + 1;
    }
}
__global__ void k_bc(DT T, const int32_t* bcidx, double* bc_prim, float* bc_hl) {
    const int fi = blockIdx.x * blockDim.x + threadIdx.x;
    if (fi >= T.NFACE || T.fkind[fi] != KG_FACE_DOMAIN) return;
    const int b = bcidx[fi];
    for (int e = 0; e < MAXW; ++e) {
        const double v = e < T.D + 2 ? T.fbc[(size_t)fi * (T.D + 2) + e] : 0.0;
        bc_prim[(size_t)b * MAXW + e] = v;
        bc_hl[(size_t)b * 2 * MAXW + e] = (float)v;
        bc_hl[(size_t)b * 2 * MAXW + MAXW + e] = (float)(v - (double)(float)v);
    }
}

// the incidence of key (2 face + role) for its cell, in the merged form of one problem
__device__ Incidence make_inc(const DT& T, int key, const int32_t* bcidx) {
    const int fi = key >> 1, role = key & 1, D = T.D;
    Incidence a;
    memset(&a, 0, sizeof(Incidence));
    const int dir = T.fdir[fi], here = T.fhere[fi];
    const double rot = T.frot[fi], area = T.farea[fi];
    for (int d = 0; d < D; ++d) { a.fmid[d] = T.fmid[(size_t)fi * D + d]; a.my_mid[d] = T.mid[(size_t)here * D + d]; }
    a.dir = (int8_t)dir;
    if (T.fkind[fi] == KG_FACE_DOMAIN) {
        a.kind = INC_DOMAIN; a.bc_kind = T.fbck[fi]; a.other = -1; a.pair = -1; a.here_side = 1;
        a.orient = rot; a.sarea = area;
        a.bc = bcidx[fi];
    } else {
        const int od = d_data_of(T, T.fthere[fi]);
        const bool solid = T.dbe[od] < 0;
        a.kind = solid ? INC_SOLID : INC_INNER;
        a.other = od; a.here_side = 1; a.orient = rot; a.sarea = area;
        for (int d = 0; d < D; ++d) { a.ot_mid[d] = T.ftmid[(size_t)fi * D + d]; a.ot_ds[d] = T.dds[(size_t)od * MAXD + d]; }
        bool ok = true;
        a.pair = d_pair(T, T.grid[here], T.dgrid[od], here, &ok);
        if (solid && od >= T.NC) {
            a.wallrec = 1;
            a.pert = a.ot_mid[dir] - T.waux[(size_t)(od - T.NC) * D + dir];
        }
        if (role == 1) {
            // the there side receives the same flux with the opposite sign
            Incidence b;
            memset(&b, 0, sizeof(Incidence));
            b.kind = INC_INNER; b.dir = (int8_t)dir; b.other = here; b.here_side = 0;
            b.orient = -rot; b.sarea = -area;
            for (int d = 0; d < D; ++d) {
                b.fmid[d] = a.fmid[d];
                b.my_mid[d] = a.ot_mid[d];
                b.ot_mid[d] = a.my_mid[d];
                b.ot_ds[d] = T.ds[(size_t)here * D + d];
            }
            b.pair = d_pair(T, T.grid[od], T.grid[here], od, &ok);
            a = b;
        }
    }
    // the fields resolved when the problems are merged (one problem at data and f base 0)
    if (a.other >= 0) {
        a.ofoff = T.foff[a.other];
        a.onv = T.dnv[a.other];
        a.ogo = (int32_t)T.g_off[T.dgrid[a.other]];
    } else {
        a.ofoff = -1; a.onv = 0; a.ogo = 0;
    }
    for (int d = 0; d < MAXD; ++d) {
        a.dxm_f[d] = (float)(a.fmid[d] - a.my_mid[d]);
        a.dxo_f[d] = (float)(a.fmid[d] - a.ot_mid[d]);
        a.ods_f[d] = (float)a.ot_ds[d];
    }
    a.orient_f = (float)a.orient;
    a.sarea_f = (float)a.sarea;
    a.pert_f = (float)a.pert;
    return a;
}

// per fluid cell: its incidences in face order, the regular-cell test, its flux record and the
// faces of a regular cell
__global__ void k_inc_build(DT T, const int32_t* fluid, int nfl, int slot, const int32_t* pref, const int32_t* keys,
                            const int32_t* bcidx, Incidence* inc, int32_t* inc_off, uint8_t* freg, FluxCell* fcrec,
                            RegRec* regrec, int* maxes) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nfl) return;
    const int i = fluid[q], D = T.D;
    const int o = pref[i], ni = pref[i + 1] - o;
    atomicMax(&maxes[0], ni);
    if (ni > MAX_INC) return;   // the host refuses the layout (more incidences than supported)
    int kk[MAX_INC];
    for (int r = 0; r < ni; ++r) {
        const int v = keys[o + r];
        int j = r;
        while (j > 0 && kk[j - 1] > v) { kk[j] = kk[j - 1]; --j; }
        kk[j] = v;
    }
    int nbcm = 0;
    bool reg = ni == 2 * D;
    int seen[2 * MAXD] = {0, 0, 0, 0, 0, 0};
    RegRec rr;
    memset(&rr, 0, sizeof(RegRec));
    for (int r = 0; r < ni; ++r) {
        const Incidence a = make_inc(T, kk[r], bcidx);
        inc[o + r] = a;
        if (a.kind == INC_DOMAIN && (a.bc_kind == KG_BC_MAXWELL || a.bc_kind == KG_BC_INFLOW)) ++nbcm;
        if (reg) {
            // per direction one face at -ds/2 and one at +ds/2, each an inner face to a
            // same-sized fluid neighbour on this cell's velocity grid
            const int d = a.dir;
            const double h = 0.5 * T.ds[(size_t)i * D + d];
            const double dm = a.fmid[d] - a.my_mid[d], dox = a.fmid[d] - a.ot_mid[d];
            reg = a.kind == INC_INNER && a.pair < 0 && a.other >= 0 && a.other < T.NC &&
                  fabs(fabs(dm) - h) <= 1e-12 * h && fabs(dox + dm) <= 1e-12 * h && a.orient * dm < 0.0;
            for (int e = 0; reg && e < D; ++e) {
                if (e != d && (fabs(a.fmid[e] - a.my_mid[e]) > 1e-12 * h || fabs(a.fmid[e] - a.ot_mid[e]) > 1e-12 * h)) reg = false;
                if (a.ot_ds[e] != T.ds[(size_t)i * D + e]) reg = false;
            }
            if (reg) ++seen[2 * d + (dm > 0.0 ? 1 : 0)];
        }
    }
    for (int e = 0; reg && e < 2 * D; ++e) reg = seen[e] == 1;
    if (reg) {
        for (int r = 0; r < ni; ++r) {
            const Incidence& a = inc[o + r];
            const int d = a.dir;
            const double dm = a.fmid[d] - a.my_mid[d];
            const int side = 2 * d + (dm > 0.0 ? 1 : 0);
            rr.nfo[side] = a.ofoff;
            rr.dxm[side] = dm;
            rr.sa[side] = a.sarea;
            rr.dxm_f[side] = a.dxm_f[d];
            rr.sa_f[side] = a.sarea_f;
            rr.nd[side] = a.other;
        }
    }
    regrec[q] = rr;
    freg[q] = reg ? 1 : 0;
    inc_off[q] = o;
    if (q == nfl - 1) inc_off[nfl] = pref[T.NC];
    FluxCell fc;
    memset(&fc, 0, sizeof(FluxCell));
    fc.foff = T.foff[i];
    fc.goff = T.g_off[T.dgrid[i]];
    fc.invV = T.dinvv[i];
    for (int d = 0; d < MAXD; ++d) fc.ds[d] = T.dds[(size_t)i * MAXD + d];
    fc.cell = i; fc.slot = slot;
    fc.inc0 = o; fc.ninc = ni;
    fc.nv = T.dnv[i]; fc.gid = T.dgrid[i]; fc.reg = reg ? 1 : 0;
    fcrec[q] = fc;
    atomicMax(&maxes[1], nbcm);
}

// per pass-cell entry (final order): its slope record
__global__ void k_screc(DT T, const int32_t* pcells, int npc, const int32_t* cell_op, const SlopeOp* ops,
                        const NbrRef* nbr, SlopeCell* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npc) return;
    const int m = pcells[k];
    SlopeCell c;
    memset(&c, 0, sizeof(SlopeCell));
    c.foff = T.foff[m];
    c.nv = T.dnv[m];
    bool reg = true;
    for (int d = 0; d < T.D && reg; ++d) {
        const SlopeOp op = ops[cell_op[k] + d];
        reg = op.kind == SLOPE_TWO && op.cntA == 1 && op.cntB == 1 && !op.projA && !op.projB;
        if (!reg) break;
        const NbrRef a = nbr[op.listA], b = nbr[op.listB];
        reg = a.pair < 0 && b.pair < 0 && T.dnv[a.data] == c.nv && T.dnv[b.data] == c.nv;
        c.nfoff[2 * d] = T.foff[a.data];
        c.nfoff[2 * d + 1] = T.foff[b.data];
        c.inv_d[2 * d] = op.inv_dsA;
        c.inv_d[2 * d + 1] = op.inv_dsB;
        c.inv_f[2 * d] = (float)op.inv_dsA;
        c.inv_f[2 * d + 1] = (float)op.inv_dsB;
    }
    c.regular = reg ? 1 : 0;
    out[k] = c;
}

// ---- slopes in the flux kernel (R2 records, 2D layouts of the packed kernel) -----------------
__global__ void k_maps(const int32_t* pcells, int npc, const int32_t* fluid, int nfl, int32_t* dsc, int32_t* dfl) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < npc) dsc[pcells[k]] = k;
    if (k < nfl) dfl[fluid[k]] = k;
}
__global__ void k_r2(const int32_t* fluid, int nfl, int dcap, const uint8_t* freg, const RegRec* regrec,
                     const SlopeCell* screc, const int32_t* dsc, const int32_t* dfl, R2Rec* r2rec, uint8_t* r2) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nfl) return;
    auto slope_reg = [&](int32_t m) { return m >= 0 && m < dcap && dsc[m] >= 0 && screc[dsc[m]].regular; };
    R2Rec r;
    memset(&r, 0, sizeof(R2Rec));
    const int32_t m = fluid[q];
    uint8_t flag = 0;
    if (freg[q] && slope_reg(m)) {
        const RegRec& rr = regrec[q];
        const SlopeCell& me = screc[dsc[m]];
        bool ok = true;
        for (int sd = 0; sd < 4 && ok; ++sd) {
            const int32_t n = rr.nd[sd];
            ok = n >= 0 && n < dcap && dfl[n] >= 0 && freg[dfl[n]] && slope_reg(n) && me.nfoff[sd] == rr.nfo[sd];
        }
        if (ok) {
            for (int t = 0; t < 4; ++t) r.sinv[t] = me.inv_f[t];
            for (int sd = 0; sd < 4; ++sd) {
                const SlopeCell& nb = screc[dsc[rr.nd[sd]]];
                for (int t = 0; t < 4; ++t) { r.nn[sd][t] = nb.nfoff[t]; r.ninv[sd][t] = nb.inv_f[t]; }
            }
            flag = 1;
        }
    }
    r2rec[q] = r;
    r2[q] = flag;
}
__global__ void k_r2_interior(int nfl, const RegRec* regrec, const int32_t* dfl, uint8_t* r2) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nfl || !r2[q]) return;
    bool interior = true;
    for (int sd = 0; sd < 4 && interior; ++sd) interior = r2[dfl[regrec[q].nd[sd]]] != 0;
    if (interior) r2[q] = 2;
}

const char* df_message(int code) {
    switch (code) {
    case DF_BOTH_BOUNDARY: return "a fluid cell has domain boundaries on both sides of a direction (no reference method)";
    case DF_BAD_STATE: return "invalid neighbour state";
    case DF_LIST_NOTHING: return "slope list references nothing / inside-solid data";
    case DF_LIST_LONG: return "a cell's slope neighbour lists exceed 24 entries (not 2:1 balanced)";
    case DF_PAIR: return "velocity pairing missing for a referenced grid pair";
    default: return "device layout build failed";
    }
}

inline int grid_of(int n, int b = 256) { return std::max(1, (n + b - 1) / b); }

// bump allocator over one device allocation
struct Bump {
    char* base;
    size_t used, cap;
    template <typename T> T* take(size_t n) {
        const size_t b = (std::max<size_t>(n, 1) * sizeof(T) + 255) / 256 * 256;
        T* p = reinterpret_cast<T*>(base + used);
        used += b;
        return p;
    }
};
template <typename T> size_t bytes_of(size_t n) { return (std::max<size_t>(n, 1) * sizeof(T) + 255) / 256 * 256; }

}  // namespace

void DevScratch::release() {
    if (dev) cudaFree(dev);
    if (pin) cudaFreeHost(pin);
    dev = nullptr; pin = nullptr;
    dev_cap = pin_cap = 0;
}

static cudaError_t grow(DevScratch& S, size_t dev_bytes, size_t pin_bytes) {
    cudaError_t e = cudaSuccess;
    if (dev_bytes > S.dev_cap) {
        if (S.dev) cudaFree(S.dev);
        S.dev = nullptr;
        S.dev_cap = 0;
        const size_t c = dev_bytes + dev_bytes / 4;
        e = cudaMalloc(&S.dev, c);
        if (e != cudaSuccess) return e;
        S.dev_cap = c;
    }
    if (pin_bytes > S.pin_cap) {
        if (S.pin) cudaFreeHost(S.pin);
        S.pin = nullptr;
        S.pin_cap = 0;
        const size_t c = pin_bytes + pin_bytes / 4;
        e = cudaMallocHost(&S.pin, c);
        if (e != cudaSuccess) return e;
        S.pin_cap = c;
    }
    return e;
}

#define DF_CUDA(x) do { cudaError_t e__ = (x); if (e__ != cudaSuccess) { err = std::string("device layout: ") + cudaGetErrorString(e__); return KG_ERR_CUDA; } } while (0)

int device_flatten(const kg_params& prm, const kg_topology& t, int slot, cudaStream_t s, Flat& F, DevLayout& L,
                   DevScratch& S, std::string& err, double* t_ms) {
    auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](int k) {
        const auto n = std::chrono::steady_clock::now();
        if (t_ms) t_ms[k] += std::chrono::duration<double, std::milli>(n - t0).count();
        t0 = n;
    };
    PairIds pid;
    int rc = flatten_head(prm, t, F, pid, err);
    if (rc) return rc;
    if (pid.dense.empty()) { err = "device layout: more than 1024 velocity grids"; return KG_ERR_TOPOLOGY; }
    rc = flatten_checks(prm, t, F, err);
    if (rc) return rc;
    rc = flatten_ib(t, F, pid, err);
    if (rc) return rc;
    const int D = t.dim, NC = t.n_cells, NF = 2 * D, NFACE = t.n_faces, G = t.n_grids;
    // fluid cells in cell order; pass-cell entries in level order
    F.fluid_cells.clear();
    for (int i = 0; i < NC; ++i)
        if (t.cell_bound_enc[i] >= 0) F.fluid_cells.push_back(i);
    const int nfl = (int)F.fluid_cells.size();
    std::vector<int32_t> pc_level;
    std::vector<int32_t> level_off(1, 0);
    pc_level.reserve(nfl);
    {
        // counting sort of the fluid cells by level (stable in cell order)
        const int nl = pid.lmax - pid.lmin + 1;
        std::vector<int32_t> cntl((size_t)nl + 1, 0);
        for (int i : F.fluid_cells) cntl[t.cell_level[i] - pid.lmin + 1] += 1;
        for (int l = 0; l < nl; ++l) cntl[l + 1] += cntl[l];
        pc_level.resize(nfl);
        std::vector<int32_t> at(cntl.begin(), cntl.end() - 1);
        for (int i : F.fluid_cells) pc_level[at[t.cell_level[i] - pid.lmin]++] = i;
        for (int l = 0; l < nl; ++l) level_off.push_back(cntl[l + 1]);
    }
    const int npc = nfl;
    const int64_t nref = t.nbr_off[NC * NF];
    lap(0);
    // ---- one pinned block with the topology arrays and the host tables, one copy -----------
    struct Seg { const void* src; size_t n; size_t off; };
    std::vector<Seg> segs;
    size_t tot = 0;
    auto seg = [&](const void* p, size_t n) {
        segs.push_back(Seg{p, n, tot});
        const size_t o = tot;
        tot += (n + 255) / 256 * 256;
        return o;
    };
    std::vector<int32_t> entry((size_t)NC, -1);
    for (int k = 0; k < npc; ++k) entry[pc_level[k]] = k;
    const size_t o_be = seg(t.cell_bound_enc, 4 * (size_t)NC), o_lev = seg(t.cell_level, 4 * (size_t)NC),
                 o_grid = seg(t.cell_grid, 4 * (size_t)NC), o_mid = seg(t.cell_midpoint, 8 * (size_t)NC * D),
                 o_ds = seg(t.cell_ds, 8 * (size_t)NC * D), o_nst = seg(t.nbr_state, (size_t)NC * NF),
                 o_noff = seg(t.nbr_off, 4 * ((size_t)NC * NF + 1)), o_nref = seg(t.nbr_ref, 4 * (size_t)nref),
                 o_fk = seg(t.face_kind, (size_t)NFACE), o_fd = seg(t.face_dir, (size_t)NFACE),
                 o_frot = seg(t.face_rot, 8 * (size_t)NFACE), o_farea = seg(t.face_area, 8 * (size_t)NFACE),
                 o_fmid = seg(t.face_midpoint, 8 * (size_t)NFACE * D), o_fh = seg(t.face_here, 4 * (size_t)NFACE),
                 o_ft = seg(t.face_there, 4 * (size_t)NFACE), o_ftm = seg(t.face_there_midpoint, 8 * (size_t)NFACE * D),
                 o_fbk = seg(t.face_bc_kind, (size_t)NFACE), o_fbc = seg(t.face_bc, 8 * (size_t)NFACE * (D + 2)),
                 o_waux = seg(t.wall_aux_point, 8 * (size_t)t.n_walls * D),
                 o_foff = seg(F.foff.data(), 8 * F.foff.size()), o_goff = seg(F.g_off.data(), 8 * F.g_off.size()),
                 o_dgrid = seg(F.dgrid.data(), 4 * F.dgrid.size()), o_dbe = seg(F.dbe.data(), 4 * F.dbe.size()),
                 o_dnv = seg(F.dnv.data(), 4 * F.dnv.size()), o_dmid = seg(F.dmid.data(), 8 * F.dmid.size()),
                 o_dds = seg(F.dds.data(), 8 * F.dds.size()), o_dinvv = seg(F.dinvv.data(), 8 * F.dinvv.size()),
                 o_pair = seg(pid.dense.data(), 4 * pid.dense.size()),
                 o_fluid = seg(F.fluid_cells.data(), 4 * (size_t)nfl), o_pcl = seg(pc_level.data(), 4 * (size_t)npc),
                 o_entry = seg(entry.data(), 4 * (size_t)NC);
    const size_t in_bytes = tot;
    // device scratch after the inputs: counts, scans, keys, depths, flags
    Bump sc{nullptr, in_bytes, 0};
    const size_t o_scnt = sc.used; sc.take<int32_t>(npc + 1);
    const size_t o_sbase = sc.used; sc.take<int32_t>(npc + 1);
    const size_t o_ccnt = sc.used; sc.take<int32_t>(nfl + 1);
    const size_t o_cbase = sc.used; sc.take<int32_t>(nfl + 1);
    const size_t o_nper = sc.used; sc.take<int32_t>(NC + 1);
    const size_t o_pref = sc.used; sc.take<int32_t>(NC + 1);
    const size_t o_fill = sc.used; sc.take<int32_t>(NC + 1);
    const size_t o_isdom = sc.used; sc.take<int32_t>(NFACE + 1);
    const size_t o_bcidx = sc.used; sc.take<int32_t>(NFACE + 1);
    const size_t o_keys = sc.used; sc.take<int32_t>(2 * (size_t)NFACE + 1);
    const size_t o_d0 = sc.used; sc.take<int32_t>(npc + 1);
    const size_t o_d1 = sc.used; sc.take<int32_t>(npc + 1);
    const size_t o_flags = sc.used; sc.take<int32_t>(16);
    const size_t dev_bytes = sc.used;
    DF_CUDA(grow(S, dev_bytes, std::max(in_bytes, (size_t)4096)));
    char* pin = (char*)S.pin;
    for (const Seg& g : segs)
        if (g.n) std::memcpy(pin + g.off, g.src, g.n);
    char* dv = (char*)S.dev;
    DF_CUDA(cudaMemcpyAsync(dv, pin, in_bytes, cudaMemcpyHostToDevice, s));
    DF_CUDA(cudaMemsetAsync(dv + in_bytes, 0, dev_bytes - in_bytes, s));
    lap(1);
    DT T;
    T.D = D; T.NC = NC; T.NWL = t.n_walls; T.NFACE = NFACE; T.G = G; T.half = 1 << (D - 1); T.lmin = pid.lmin;
    T.be = (const int32_t*)(dv + o_be); T.lev = (const int32_t*)(dv + o_lev); T.grid = (const int32_t*)(dv + o_grid);
    T.mid = (const double*)(dv + o_mid); T.ds = (const double*)(dv + o_ds);
    T.nst = (const int8_t*)(dv + o_nst); T.noff = (const int32_t*)(dv + o_noff); T.nref = (const int32_t*)(dv + o_nref);
    T.fkind = (const int8_t*)(dv + o_fk); T.fdir = (const int8_t*)(dv + o_fd);
    T.frot = (const double*)(dv + o_frot); T.farea = (const double*)(dv + o_farea); T.fmid = (const double*)(dv + o_fmid);
    T.fhere = (const int32_t*)(dv + o_fh); T.fthere = (const int32_t*)(dv + o_ft);
    T.ftmid = (const double*)(dv + o_ftm); T.fbck = (const int8_t*)(dv + o_fbk); T.fbc = (const double*)(dv + o_fbc);
    T.waux = (const double*)(dv + o_waux);
    T.foff = (const int64_t*)(dv + o_foff); T.g_off = (const int64_t*)(dv + o_goff);
    T.dgrid = (const int32_t*)(dv + o_dgrid); T.dbe = (const int32_t*)(dv + o_dbe); T.dnv = (const int32_t*)(dv + o_dnv);
    T.dmid = (const double*)(dv + o_dmid); T.dds = (const double*)(dv + o_dds); T.dinvv = (const double*)(dv + o_dinvv);
    T.pair = (const int32_t*)(dv + o_pair);
    int* flags = (int*)(dv + o_flags);
    T.err = flags;                       // flags[0..1]: error code, item
    int* maxes = flags + 4;              // [max incidences, max Maxwellian-state faces]
    int* dflags = flags + 8;             // depth sweep: changed, not earlier
    const int32_t* fluid_d = (const int32_t*)(dv + o_fluid);
    const int32_t* pcl_d = (const int32_t*)(dv + o_pcl);
    const int32_t* entry_d = (const int32_t*)(dv + o_entry);
    int32_t* scnt = (int32_t*)(dv + o_scnt);
    int32_t* sbase = (int32_t*)(dv + o_sbase);
    int32_t* ccnt = (int32_t*)(dv + o_ccnt);
    int32_t* cbase = (int32_t*)(dv + o_cbase);
    int32_t* nper = (int32_t*)(dv + o_nper);
    int32_t* pref = (int32_t*)(dv + o_pref);
    int32_t* fillc = (int32_t*)(dv + o_fill);
    int32_t* isdom = (int32_t*)(dv + o_isdom);
    int32_t* bcidx = (int32_t*)(dv + o_bcidx);
    int32_t* keys = (int32_t*)(dv + o_keys);
    int32_t* d0 = (int32_t*)(dv + o_d0);
    int32_t* d1 = (int32_t*)(dv + o_d1);

    // ---- counts and their prefix sums ----------------------------------------------------
    k_slope_count<<<grid_of(npc), 256, 0, s>>>(T, pcl_d, npc, scnt);
    k_scan<<<1, 1024, 0, s>>>(scnt, npc, sbase);
    k_crit_count<<<grid_of(nfl), 256, 0, s>>>(T, fluid_d, nfl, ccnt);
    k_scan<<<1, 1024, 0, s>>>(ccnt, nfl, cbase);
    if (NFACE > 0) k_inc_count<<<grid_of(NFACE), 256, 0, s>>>(T, nper, isdom);
    k_scan<<<1, 1024, 0, s>>>(nper, NC, pref);
    k_scan<<<1, 1024, 0, s>>>(isdom, NFACE, bcidx);
    DF_CUDA(cudaGetLastError());
    int32_t tots[6];
    DF_CUDA(cudaMemcpyAsync(&tots[0], sbase + npc, 4, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaMemcpyAsync(&tots[1], cbase + nfl, 4, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaMemcpyAsync(&tots[2], pref + NC, 4, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaMemcpyAsync(&tots[3], bcidx + NFACE, 4, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaMemcpyAsync(&tots[4], flags, 8, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaStreamSynchronize(s));
    if (tots[4]) { err = df_message(tots[4]); return KG_ERR_TOPOLOGY; }
    lap(2);
    const int nsn = tots[0], ncn = tots[1], ninc = tots[2], nbc = tots[3];
    // ---- the layout's arrays ---------------------------------------------------------------
    size_t lb = bytes_of<SlopeOp>((size_t)npc * D) + bytes_of<NbrRef>(nsn) + 3 * bytes_of<int32_t>(npc) +
                bytes_of<SlopeCell>(npc) + bytes_of<CritOp>((size_t)nfl * D) + bytes_of<int32_t>(ncn) +
                bytes_of<int32_t>(nfl + 1) + bytes_of<Incidence>(ninc) + bytes_of<double>((size_t)nbc * MAXW) +
                bytes_of<float>((size_t)nbc * 2 * MAXW) + 2 * bytes_of<uint8_t>(nfl) + bytes_of<FluxCell>(nfl) +
                bytes_of<RegRec>(nfl) + bytes_of<R2Rec>(nfl) + 2 * bytes_of<int32_t>(F.n_data) + bytes_of<int32_t>(nfl) +
                bytes_of<int32_t>(npc + 1);
    L.release();
    {
        void* a = nullptr;
        DF_CUDA(cudaMalloc(&a, lb));
        L.arena = std::shared_ptr<void>(a, [](void* p) { cudaFree(p); });
    }
    L.bytes = lb;
    Bump b{(char*)L.arena.get(), 0, lb};
    L.slope_ops = b.take<SlopeOp>((size_t)npc * D);
    L.slope_nbr = b.take<NbrRef>(nsn);
    L.cell_slope_op = b.take<int32_t>(npc);
    L.pass_cells = b.take<int32_t>(npc);
    int32_t* cell_op_level = b.take<int32_t>(npc);
    L.screc = b.take<SlopeCell>(npc);
    L.crit_ops = b.take<CritOp>((size_t)nfl * D);
    L.crit_nbr = b.take<int32_t>(ncn);
    L.inc_off = b.take<int32_t>(nfl + 1);
    L.inc = b.take<Incidence>(ninc);
    L.bc_prim = b.take<double>((size_t)nbc * MAXW);
    L.bc_hl = b.take<float>((size_t)nbc * 2 * MAXW);
    L.fluid_reg = b.take<uint8_t>(nfl);
    L.fluid_r2 = b.take<uint8_t>(nfl);
    L.fcrec = b.take<FluxCell>(nfl);
    L.regrec = b.take<RegRec>(nfl);
    L.r2rec = b.take<R2Rec>(nfl);
    L.fluid_cells = b.take<int32_t>(nfl);
    L.dsc = b.take<int32_t>(F.n_data);
    L.dfl = b.take<int32_t>(F.n_data);
    int32_t* offs_d = b.take<int32_t>(npc + 1);
    L.n_slope_ops = (int64_t)npc * D; L.n_slope_nbr = nsn; L.n_pass = npc; L.n_crit_ops = (int64_t)nfl * D;
    L.n_crit_nbr = ncn; L.n_fluid = nfl; L.n_inc = ninc; L.n_bc = nbc; L.n_data = F.n_data;
    DF_CUDA(cudaMemsetAsync(L.arena.get(), 0, lb, s));
    DF_CUDA(cudaMemcpyAsync(L.fluid_cells, fluid_d, 4 * (size_t)nfl, cudaMemcpyDeviceToDevice, s));
    // ---- fills -------------------------------------------------------------------------------
    k_slope_fill<<<grid_of(npc), 256, 0, s>>>(T, pcl_d, npc, sbase, L.slope_ops, L.slope_nbr, cell_op_level);
    k_crit_fill<<<grid_of(nfl), 256, 0, s>>>(T, fluid_d, nfl, cbase, L.crit_ops, L.crit_nbr);
    if (NFACE > 0) {
        k_inc_place<<<grid_of(NFACE), 256, 0, s>>>(T, pref, fillc, keys);
        k_bc<<<grid_of(NFACE), 256, 0, s>>>(T, bcidx, L.bc_prim, L.bc_hl);
    }
    k_inc_build<<<grid_of(nfl, 128), 128, 0, s>>>(T, fluid_d, nfl, slot, pref, keys, bcidx, L.inc, L.inc_off, L.fluid_reg,
                                             L.fcrec, L.regrec, maxes);
    DF_CUDA(cudaGetLastError());
    // ---- slope passes by dependency depth ------------------------------------------------------
    bool ok_depth = true;
    int maxd = 0;
    {
        int32_t* din = d0;
        int32_t* dout = d1;
        for (int it = 0; it <= npc + 1; ++it) {
            DF_CUDA(cudaMemsetAsync(dflags, 0, 8, s));
            k_depth<<<grid_of(npc), 256, 0, s>>>(T, L.slope_ops, L.slope_nbr, entry_d, npc, din, dout, dflags);
            int hf[2];
            DF_CUDA(cudaMemcpyAsync(hf, dflags, 8, cudaMemcpyDeviceToHost, s));
            DF_CUDA(cudaStreamSynchronize(s));
            std::swap(din, dout);
            if (hf[1]) { ok_depth = false; break; }
            if (!hf[0]) break;
        }
        if (ok_depth) {
            std::vector<int32_t> dh(npc);
            DF_CUDA(cudaMemcpyAsync(dh.data(), din, 4 * (size_t)npc, cudaMemcpyDeviceToHost, s));
            DF_CUDA(cudaStreamSynchronize(s));
            for (int32_t v : dh) maxd = std::max(maxd, (int)v);
            k_partition<<<1, 1024, 0, s>>>(din, npc, maxd, pcl_d, L.pass_cells, L.cell_slope_op, offs_d, D);
        }
    }
    F.pass_cells_off.clear();
    if (ok_depth) {
        std::vector<int32_t> offs((size_t)maxd + 2);
        DF_CUDA(cudaMemcpyAsync(offs.data(), offs_d, 4 * offs.size(), cudaMemcpyDeviceToHost, s));
        F.pass_cells.resize(npc);
        DF_CUDA(cudaMemcpyAsync(F.pass_cells.data(), L.pass_cells, 4 * (size_t)npc, cudaMemcpyDeviceToHost, s));
        DF_CUDA(cudaStreamSynchronize(s));
        F.pass_cells_off.assign(offs.begin(), offs.end());
    } else {
        // one pass per level, in level order
        DF_CUDA(cudaMemcpyAsync(L.pass_cells, pcl_d, 4 * (size_t)npc, cudaMemcpyDeviceToDevice, s));
        DF_CUDA(cudaMemcpyAsync(L.cell_slope_op, cell_op_level, 4 * (size_t)npc, cudaMemcpyDeviceToDevice, s));
        F.pass_cells = pc_level;
        F.pass_cells_off = level_off;
    }
    k_screc<<<grid_of(npc, 128), 128, 0, s>>>(T, L.pass_cells, npc, L.cell_slope_op, L.slope_ops, L.slope_nbr, L.screc);
    DF_CUDA(cudaGetLastError());
    F.fluid_reg.resize(nfl);
    int hm[4];
    DF_CUDA(cudaMemcpyAsync(F.fluid_reg.data(), L.fluid_reg, (size_t)nfl, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaMemcpyAsync(hm, maxes, 8, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaMemcpyAsync(hm + 2, flags, 8, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaStreamSynchronize(s));
    if (hm[2]) { err = df_message(hm[2]); return KG_ERR_TOPOLOGY; }
    F.max_inc = hm[0];
    F.max_bcm = hm[1];
    F.devlay = true;
    lap(3);
    if (F.p_j0.empty()) { F.p_j0.push_back(0); F.p_cnt.push_back(0); }
    return KG_OK;
}

int device_r2(const Flat& M, DevLayout& L, bool fuse, cudaStream_t s, std::vector<uint8_t>& r2, std::string& err) {
    const int nfl = (int)L.n_fluid, npc = (int)L.n_pass;
    r2.assign((size_t)nfl, 0);
    if (!fuse || M.dim != 2) {
        DF_CUDA(cudaMemsetAsync(L.r2rec, 0, sizeof(R2Rec) * std::max(nfl, 1), s));
        DF_CUDA(cudaMemsetAsync(L.fluid_r2, 0, std::max(nfl, 1), s));
        return KG_OK;
    }
    DF_CUDA(cudaMemsetAsync(L.dsc, 0xff, 4 * (size_t)L.n_data, s));
    DF_CUDA(cudaMemsetAsync(L.dfl, 0xff, 4 * (size_t)L.n_data, s));
    const int32_t* fluid = L.fluid_cells;
    k_maps<<<grid_of(std::max(npc, nfl)), 256, 0, s>>>(L.pass_cells, npc, fluid, nfl, L.dsc, L.dfl);
    k_r2<<<grid_of(nfl, 128), 128, 0, s>>>(fluid, nfl, (int)L.n_data, L.fluid_reg, L.regrec, L.screc, L.dsc, L.dfl, L.r2rec,
                                      L.fluid_r2);
    k_r2_interior<<<grid_of(nfl), 256, 0, s>>>(nfl, L.regrec, L.dfl, L.fluid_r2);
    DF_CUDA(cudaGetLastError());
    DF_CUDA(cudaMemcpyAsync(r2.data(), L.fluid_r2, (size_t)nfl, cudaMemcpyDeviceToHost, s));
    DF_CUDA(cudaStreamSynchronize(s));
    return KG_OK;
}

}  // namespace kg

// ---- merging device-built layouts (a batch of problems) ------------------------------------
namespace kg {
namespace {

__global__ void k_m_slope_ops(const SlopeOp* in, int64_t n, SlopeOp* out, int32_t dbase, int32_t snb) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    SlopeOp op = in[i];
    op.cell += dbase;
    op.listA += snb;
    op.listB += snb;
    out[i] = op;
}
__global__ void k_m_nbr(const NbrRef* in, int64_t n, NbrRef* out, int32_t dbase, int32_t pairacc) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    NbrRef r = in[i];
    r.data += dbase;
    r.pair = r.pair >= 0 ? r.pair + pairacc : r.pair;
    out[i] = r;
}
__global__ void k_m_crit(const CritOp* in, int64_t n, CritOp* out, int32_t cacc) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    CritOp op = in[i];
    op.listA += cacc;
    op.listB += cacc;
    out[i] = op;
}
__global__ void k_m_crit_nbr(const int32_t* in, int64_t n, int32_t* out, int32_t dbase) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i] >= 0 ? in[i] + dbase : -1;
}
__global__ void k_m_inc(const Incidence* in, int64_t n, Incidence* out, int32_t dbase, int64_t fbase, int64_t PGacc,
                        int32_t pairacc, int32_t bcacc) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    Incidence a = in[i];
    if (a.other >= 0) {
        a.other += dbase;
        a.ofoff += fbase;
        a.ogo += (int32_t)PGacc;
    }
    a.pair = a.pair >= 0 ? a.pair + pairacc : a.pair;
    a.bc += bcacc;
    out[i] = a;
}
// per fluid-list entry: the cell, the regular flag, the incidence range end, the flux record and
// the regular cell's faces, at their merged positions
__global__ void k_m_fluid(const int32_t* cells, const uint8_t* reg, const int32_t* inc_off, const FluxCell* fc,
                          const RegRec* rr, int n, int32_t* cells_o, uint8_t* reg_o, int32_t* inc_off_o, FluxCell* fc_o,
                          RegRec* rr_o, int32_t dbase, int64_t fbase, int64_t PGacc, int32_t incacc, int32_t Gacc, int D) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    cells_o[q] = cells[q] + dbase;
    reg_o[q] = reg[q];
    inc_off_o[q + 1] = inc_off[q + 1] + incacc;
    FluxCell c = fc[q];
    c.foff += fbase;
    c.goff += PGacc;
    c.cell += dbase;
    c.inc0 += incacc;
    c.gid += Gacc;
    fc_o[q] = c;
    RegRec r = rr[q];
    if (reg[q]) {
        for (int s = 0; s < 2 * D; ++s) { r.nfo[s] += fbase; r.nd[s] += dbase; }
    }
    rr_o[q] = r;
}
// one part's pass-cell entries into the merged pass order: entry k of pass p goes to
// base[p] + k - off[p]
__global__ void k_m_pass(const int32_t* pc, const int32_t* cop, int npc, const int32_t* off, const int32_t* base,
                         int npass, int32_t* pc_o, int32_t* cop_o, int32_t dbase, int32_t sops) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npc) return;
    int p = 0;
    while (p + 1 < npass && off[p + 1] <= k) ++p;
    const int m = base[p] + k - off[p];
    pc_o[m] = pc[k] + dbase;
    cop_o[m] = cop[k] + sops;
}

}  // namespace

int device_merge(const std::vector<MergeIn>& parts, int64_t n_data, int64_t npc_total, const int64_t* foff,
                 const int32_t* dnv, int D, cudaStream_t s, DevLayout& M, DevScratch& S, std::string& err) {
    int64_t nso = 0, nsn = 0, ncop = 0, ncn = 0, nfl = 0, ninc = 0, nbc = 0;
    size_t tab = 0;
    for (const MergeIn& p : parts) {
        const DevLayout& L = *p.L;
        nso += L.n_slope_ops; nsn += L.n_slope_nbr; ncop += L.n_crit_ops; ncn += L.n_crit_nbr;
        nfl += L.n_fluid; ninc += L.n_inc; nbc += L.n_bc;
        tab += 2 * p.pass_off.size();
    }
    size_t lb = bytes_of<SlopeOp>(nso) + bytes_of<NbrRef>(nsn) + 3 * bytes_of<int32_t>(npc_total) +
                bytes_of<SlopeCell>(npc_total) + bytes_of<CritOp>(ncop) + bytes_of<int32_t>(ncn) +
                bytes_of<int32_t>(nfl + 1) + bytes_of<Incidence>(ninc) + bytes_of<double>(nbc * MAXW) +
                bytes_of<float>(nbc * 2 * MAXW) + 2 * bytes_of<uint8_t>(nfl) + bytes_of<FluxCell>(nfl) +
                bytes_of<RegRec>(nfl) + bytes_of<R2Rec>(nfl) + 2 * bytes_of<int32_t>(n_data) + bytes_of<int32_t>(nfl) +
                bytes_of<int64_t>(n_data + 1) + bytes_of<int32_t>(n_data);
    M.release();
    {
        void* a = nullptr;
        DF_CUDA(cudaMalloc(&a, lb));
        M.arena = std::shared_ptr<void>(a, [](void* p) { cudaFree(p); });
    }
    M.bytes = lb;
    Bump b{(char*)M.arena.get(), 0, lb};
    M.slope_ops = b.take<SlopeOp>(nso);
    M.slope_nbr = b.take<NbrRef>(nsn);
    M.cell_slope_op = b.take<int32_t>(npc_total);
    M.pass_cells = b.take<int32_t>(npc_total);
    b.take<int32_t>(npc_total);
    M.screc = b.take<SlopeCell>(npc_total);
    M.crit_ops = b.take<CritOp>(ncop);
    M.crit_nbr = b.take<int32_t>(ncn);
    M.inc_off = b.take<int32_t>(nfl + 1);
    M.inc = b.take<Incidence>(ninc);
    M.bc_prim = b.take<double>(nbc * MAXW);
    M.bc_hl = b.take<float>(nbc * 2 * MAXW);
    M.fluid_reg = b.take<uint8_t>(nfl);
    M.fluid_r2 = b.take<uint8_t>(nfl);
    M.fcrec = b.take<FluxCell>(nfl);
    M.regrec = b.take<RegRec>(nfl);
    M.r2rec = b.take<R2Rec>(nfl);
    M.fluid_cells = b.take<int32_t>(nfl);
    M.dsc = b.take<int32_t>(n_data);
    M.dfl = b.take<int32_t>(n_data);
    int64_t* d_foff = b.take<int64_t>(n_data + 1);
    int32_t* d_dnv = b.take<int32_t>(n_data);
    M.n_slope_ops = nso; M.n_slope_nbr = nsn; M.n_pass = npc_total; M.n_crit_ops = ncop; M.n_crit_nbr = ncn;
    M.n_fluid = nfl; M.n_inc = ninc; M.n_bc = nbc; M.n_data = n_data;
    DF_CUDA(cudaMemsetAsync(M.arena.get(), 0, lb, s));
    DF_CUDA(cudaMemcpyAsync(d_foff, foff, sizeof(int64_t) * (n_data + 1), cudaMemcpyHostToDevice, s));
    DF_CUDA(cudaMemcpyAsync(d_dnv, dnv, sizeof(int32_t) * n_data, cudaMemcpyHostToDevice, s));
    // the per-part pass tables (local pass offsets, merged bases) through the pinned scratch
    DF_CUDA(grow(S, std::max<size_t>(4 * tab, 256), std::max<size_t>(4 * tab, 256)));
    int32_t* pin = (int32_t*)S.pin;
    {
        size_t at = 0;
        for (const MergeIn& p : parts) {
            for (size_t i = 0; i < p.pass_off.size(); ++i) pin[at + i] = p.pass_off[i];
            for (size_t i = 0; i < p.pass_base.size(); ++i) pin[at + p.pass_off.size() + i] = p.pass_base[i];
            at += 2 * p.pass_off.size();
        }
        if (tab) DF_CUDA(cudaMemcpyAsync(S.dev, pin, 4 * tab, cudaMemcpyHostToDevice, s));
    }
    int64_t so = 0, sn = 0, co = 0, cn = 0, fl = 0, ic = 0, bc = 0;
    size_t at = 0;
    for (const MergeIn& p : parts) {
        const DevLayout& L = *p.L;
        if (L.n_slope_ops) k_m_slope_ops<<<grid_of((int)L.n_slope_ops), 256, 0, s>>>(L.slope_ops, L.n_slope_ops, M.slope_ops + so, p.dbase, p.snb);
        if (L.n_slope_nbr) k_m_nbr<<<grid_of((int)L.n_slope_nbr), 256, 0, s>>>(L.slope_nbr, L.n_slope_nbr, M.slope_nbr + sn, p.dbase, p.pairacc);
        if (L.n_crit_ops) k_m_crit<<<grid_of((int)L.n_crit_ops), 256, 0, s>>>(L.crit_ops, L.n_crit_ops, M.crit_ops + co, p.cacc);
        if (L.n_crit_nbr) k_m_crit_nbr<<<grid_of((int)L.n_crit_nbr), 256, 0, s>>>(L.crit_nbr, L.n_crit_nbr, M.crit_nbr + cn, p.dbase);
        if (L.n_inc) k_m_inc<<<grid_of((int)L.n_inc), 256, 0, s>>>(L.inc, L.n_inc, M.inc + ic, p.dbase, p.fbase, p.PGacc, p.pairacc, p.bcacc);
        if (L.n_fluid)
            k_m_fluid<<<grid_of((int)L.n_fluid, 128), 128, 0, s>>>(L.fluid_cells, L.fluid_reg, L.inc_off, L.fcrec, L.regrec, (int)L.n_fluid,
                                                             M.fluid_cells + fl, M.fluid_reg + fl, M.inc_off + fl, M.fcrec + fl,
                                                             M.regrec + fl, p.dbase, p.fbase, p.PGacc, p.incacc, p.Gacc, D);
        if (L.n_bc) {
            DF_CUDA(cudaMemcpyAsync(M.bc_prim + bc * MAXW, L.bc_prim, sizeof(double) * L.n_bc * MAXW, cudaMemcpyDeviceToDevice, s));
            DF_CUDA(cudaMemcpyAsync(M.bc_hl + bc * 2 * MAXW, L.bc_hl, sizeof(float) * L.n_bc * 2 * MAXW, cudaMemcpyDeviceToDevice, s));
        }
        if (L.n_pass) {
            const int32_t* off = (const int32_t*)S.dev + at;
            const int32_t* base = off + p.pass_off.size();
            k_m_pass<<<grid_of((int)L.n_pass), 256, 0, s>>>(L.pass_cells, L.cell_slope_op, (int)L.n_pass, off, base,
                                                          (int)p.pass_base.size(), M.pass_cells, M.cell_slope_op, p.dbase, p.sops);
        }
        at += 2 * p.pass_off.size();
        so += L.n_slope_ops; sn += L.n_slope_nbr; co += L.n_crit_ops; cn += L.n_crit_nbr;
        fl += L.n_fluid; ic += L.n_inc; bc += L.n_bc;
    }
    // the slope records from the merged arrays
    DT T;
    std::memset(&T, 0, sizeof(DT));
    T.D = D;
    T.foff = d_foff;
    T.dnv = d_dnv;
    if (npc_total)
        k_screc<<<grid_of((int)npc_total, 128), 128, 0, s>>>(T, M.pass_cells, (int)npc_total, M.cell_slope_op, M.slope_ops,
                                                            M.slope_nbr, M.screc);
    DF_CUDA(cudaGetLastError());
    DF_CUDA(cudaStreamSynchronize(s));   // the pinned tables are read by the copy above
    return KG_OK;
}

}  // namespace kg
