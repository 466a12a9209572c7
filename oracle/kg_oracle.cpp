// kg_oracle.cpp -- CPU restatement of KitAMR.jl's per-step phase-space path, in FP64.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity checker for libkitgpu.so and
// the timed CPU baseline of bench.py; nothing in the product links or calls it.
//
// It follows the reference's own data flow: per-face scatter of micro/macro fluxes
// with the reference's level merge walks, the coarse-to-fine slope sweep with the
// transverse correction, the IB solid-cell extrapolation and diffuse-wall update,
// and the CAIDVM / Euler marching.  Each function cites the reference (paths
// relative to the KitAMR.jl project).  Parity with the reference itself is
// UNPINNED by the reference's tests (test/runtests.jl asserts nothing and the
// reference ships no golden vectors; no Julia exists here); it is pinned instead by
// the physics known-answer tests in tests/test_oracle_kat.py.
//
// Input is the reference-shaped kg_topology of include/kitgpu.h.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/kitgpu.h"

namespace {

constexpr double EPS_REF = 1e-12;                  // src/Abstract/Types.jl:3
constexpr double JL_EPS = 2.220446049250313e-16;   // Julia eps() = eps(Float64)
constexpr double PI = 3.141592653589793;

thread_local std::string g_err;

struct Grid {
    int64_t off = 0;
    int nv = 0;
    const int8_t* level = nullptr;
    const double* weight = nullptr;
    const double* mid = nullptr;  // column-major nv x dim
    double u(int i, int d) const { return mid[(size_t)d * nv + i]; }
};

// A PsData-like view of anything that holds velocity data (cell or SolidNeighbor).
struct Data {
    int kind = 0;            // 0 none, 1 cell, 2 wall, 3 inside-solid
    int idx = -1;
};

struct Model {
    int dim = 2, ndf = 2;
    kg_params prm{};
    const kg_topology* t = nullptr;
    std::vector<Grid> grids;
    // per cell
    std::vector<int64_t> foff;           // f offset (in doubles)
    std::vector<int64_t> soff;           // sdf offset (in doubles)
    std::vector<double> vsflux;          // same layout as f (cells)
    std::vector<double> wflux;           // n_cells x (dim+2)
    // walls: own df and sdf on the donor grid
    std::vector<int64_t> wfoff, wsoff;
    std::vector<double> wall_f, wall_sdf;
    // state (pointers to caller arrays)
    double* f = nullptr;
    double* sdf = nullptr;
    double* w = nullptr;
    double* prim = nullptr;
    double* qf = nullptr;
    double dt = 0;
    int nthreads = 1;

    int nw() const { return dim + 2; }
    Data ref(int32_t r) const {
        Data d;
        if (r == KG_NBR_NONE) { d.kind = 0; }
        else if (r == KG_NBR_INSIDE) { d.kind = 3; }
        else if (r >= 0) { d.kind = 1; d.idx = r; }
        else { d.kind = 2; d.idx = -1 - r; }
        return d;
    }
    const Grid& grid_of(const Data& d) const {
        int c = d.kind == 1 ? d.idx : t->wall_donor[d.idx];
        return grids[t->cell_grid[c]];
    }
    int bound_enc(const Data& d) const {
        if (d.kind == 1) return t->cell_bound_enc[d.idx];
        return t->cell_bound_enc[t->wall_solid[d.idx]];  // SolidNeighbor.bound_enc = solid_cell.bound_enc
    }
    const double* mid(const Data& d) const {
        int c = d.kind == 1 ? d.idx : t->wall_solid[d.idx];  // SolidNeighbor.midpoint = solid_cell.midpoint
        return t->cell_midpoint + (size_t)c * dim;
    }
    const double* ds(const Data& d) const {
        int c = d.kind == 1 ? d.idx : t->wall_solid[d.idx];
        return t->cell_ds + (size_t)c * dim;
    }
    double* df(const Data& d) { return d.kind == 1 ? f + foff[d.idx] : wall_f.data() + wfoff[d.idx]; }
    double* sdfp(const Data& d) { return d.kind == 1 ? sdf + soff[d.idx] : wall_sdf.data() + wsoff[d.idx]; }
    // element accessors in the reference's column-major layouts
    static double& F(double* p, int nv, int i, int k) { return p[(size_t)k * nv + i]; }
    static double& S(double* p, int nv, int ndf, int i, int k, int d) { return p[((size_t)d * ndf + k) * nv + i]; }
    const int32_t* nbr_begin(int c, int k) const { return t->nbr_ref + t->nbr_off[c * 2 * dim + k]; }
    int nbr_count(int c, int k) const { return t->nbr_off[c * 2 * dim + k + 1] - t->nbr_off[c * 2 * dim + k]; }
    int nbr_state(int c, int k) const { return t->nbr_state[c * 2 * dim + k]; }
};

// ---------------------------------------------------------------- KitCore -------
// get_prim_2D / get_prim_3D (lib/KitCore/2D.jl:9-16, 3D.jl:12-20)
void get_prim(const Model& m, const double* w, double* prim) {
    double g = m.prm.gamma;
    prim[0] = w[0];
    if (m.dim == 2) {
        prim[1] = w[1] / w[0];
        prim[2] = w[2] / w[0];
        prim[3] = 0.5 * w[0] / (g - 1.0) / (w[3] - 0.5 * (w[1] * w[1] + w[2] * w[2]) / w[0]);
    } else {
        prim[1] = w[1] / w[0];
        prim[2] = w[2] / w[0];
        prim[3] = w[3] / w[0];
        prim[4] = 0.5 * w[0] / (g - 1.0) / (w[4] - 0.5 * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]) / w[0]);
    }
}
// discrete_maxwell_2D2F / 3D1F at one velocity (2D2F.jl:17-23, 3D1F.jl:14-23)
inline void maxwell(const Model& m, const Grid& g, int i, const double* prim, double* out) {
    if (m.dim == 2) {
        double u = g.u(i, 0), v = g.u(i, 1);
        double h = prim[0] * (prim[3] / PI) * std::exp(-prim[3] * ((u - prim[1]) * (u - prim[1]) + (v - prim[2]) * (v - prim[2])));
        out[0] = h;
        out[1] = h * m.prm.K / (2.0 * prim[3]);
    } else {
        double u = g.u(i, 0), v = g.u(i, 1), ww = g.u(i, 2);
        out[0] = prim[0] * std::pow(prim[4] / PI, 1.5) *
                 std::exp(-prim[4] * ((u - prim[1]) * (u - prim[1]) + (v - prim[2]) * (v - prim[2]) + (ww - prim[3]) * (ww - prim[3])));
    }
}
// micro_to_macro_2D2F / 3D1F over a subset (2D2F.jl:119-126, 3D1F.jl:109-123)
// `sel` chooses the velocity cells; vals are indexed by the subset position.
void moments_subset(const Model& m, const Grid& g, const std::vector<int>& sel, const std::vector<double>& vals, double* out) {
    int n = (int)sel.size();
    if (m.dim == 2) {
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (int a = 0; a < n; ++a) { int i = sel[a]; s0 += g.weight[i] * vals[a]; }
        for (int a = 0; a < n; ++a) { int i = sel[a]; s1 += g.weight[i] * g.u(i, 0) * vals[a]; }
        for (int a = 0; a < n; ++a) { int i = sel[a]; s2 += g.weight[i] * g.u(i, 1) * vals[a]; }
        for (int a = 0; a < n; ++a) {
            int i = sel[a];
            double u = g.u(i, 0), v = g.u(i, 1);
            s3 += g.weight[i] * ((u * u + v * v) * vals[a] + vals[n + a]);
        }
        out[0] = s0; out[1] = s1; out[2] = s2; out[3] = 0.5 * s3;
    } else {
        double s[5] = {0, 0, 0, 0, 0};
        for (int a = 0; a < n; ++a) { int i = sel[a]; s[0] += g.weight[i] * vals[a]; }
        for (int d = 0; d < 3; ++d)
            for (int a = 0; a < n; ++a) { int i = sel[a]; s[1 + d] += g.weight[i] * g.u(i, d) * vals[a]; }
        for (int a = 0; a < n; ++a) {
            int i = sel[a];
            double u = g.u(i, 0), v = g.u(i, 1), ww = g.u(i, 2);
            s[4] += g.weight[i] * (u * u + v * v + ww * ww) * vals[a];
        }
        out[0] = s[0]; out[1] = s[1]; out[2] = s[2]; out[3] = s[3]; out[4] = 0.5 * s[4];
    }
}
// calc_w0 over a whole grid (Theory/Math.jl:233-238; micro_to_macro_*)
void calc_w0(const Model& m, const Grid& g, const double* df, double* out) {
    int nv = g.nv;
    if (m.dim == 2) {
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (int i = 0; i < nv; ++i) s0 += g.weight[i] * df[i];
        for (int i = 0; i < nv; ++i) s1 += g.weight[i] * g.u(i, 0) * df[i];
        for (int i = 0; i < nv; ++i) s2 += g.weight[i] * g.u(i, 1) * df[i];
        for (int i = 0; i < nv; ++i) {
            double u = g.u(i, 0), v = g.u(i, 1);
            s3 += g.weight[i] * ((u * u + v * v) * df[i] + df[nv + i]);
        }
        out[0] = s0; out[1] = s1; out[2] = s2; out[3] = 0.5 * s3;
    } else {
        double s[5] = {0, 0, 0, 0, 0};
        for (int i = 0; i < nv; ++i) s[0] += g.weight[i] * df[i];
        for (int d = 0; d < 3; ++d)
            for (int i = 0; i < nv; ++i) s[1 + d] += g.weight[i] * g.u(i, d) * df[i];
        for (int i = 0; i < nv; ++i) {
            double u = g.u(i, 0), v = g.u(i, 1), ww = g.u(i, 2);
            s[4] += g.weight[i] * (u * u + v * v + ww * ww) * df[i];
        }
        out[0] = s[0]; out[1] = s[1]; out[2] = s[2]; out[3] = s[3]; out[4] = 0.5 * s[4];
    }
}
// heat_flux_2D2F / 3D1F (2D2F.jl:68-88, 3D1F.jl:41-72)
void heat_flux(const Model& m, const Grid& g, const double* df, const double* prim, double* q) {
    int nv = g.nv;
    if (m.dim == 2) {
        double a = 0, b = 0, c = 0, d = 0;
        for (int i = 0; i < nv; ++i) {
            double cu = g.u(i, 0) - prim[1], cv = g.u(i, 1) - prim[2];
            a += g.weight[i] * cu * (cu * cu + cv * cv) * df[i];
        }
        for (int i = 0; i < nv; ++i) b += g.weight[i] * (g.u(i, 0) - prim[1]) * df[nv + i];
        for (int i = 0; i < nv; ++i) {
            double cu = g.u(i, 0) - prim[1], cv = g.u(i, 1) - prim[2];
            c += g.weight[i] * cv * (cu * cu + cv * cv) * df[i];
        }
        for (int i = 0; i < nv; ++i) d += g.weight[i] * (g.u(i, 1) - prim[2]) * df[nv + i];
        q[0] = 0.5 * (a + b);
        q[1] = 0.5 * (c + d);
    } else {
        for (int k = 0; k < 3; ++k) {
            double s = 0;
            for (int i = 0; i < nv; ++i) {
                double cu = g.u(i, 0) - prim[1], cv = g.u(i, 1) - prim[2], cw = g.u(i, 2) - prim[3];
                double ck = k == 0 ? cu : (k == 1 ? cv : cw);
                s += g.weight[i] * ck * (cu * cu + cv * cv + cw * cw) * df[i];
            }
            q[k] = 0.5 * s;
        }
    }
}
// shakhov_part_2D2F / 3D1F at one velocity (2D2F.jl:22-67, 3D1F.jl:24-40)
inline void shakhov(const Model& m, const Grid& g, int i, const double* H, const double* prim, const double* qf, double* out) {
    double Pr = m.prm.Pr;
    if (m.dim == 2) {
        double K = m.prm.K;
        double cu = g.u(i, 0) - prim[1], cv = g.u(i, 1) - prim[2];
        double c2 = cu * cu + cv * cv;
        double pre = 0.8 * (1 - Pr) * prim[3] * prim[3] / prim[0] * (cu * qf[0] + cv * qf[1]);
        out[0] = pre * (2 * prim[3] * c2 + K - 5) * H[0];
        out[1] = pre * (2 * prim[3] * c2 + K - 3) * H[1];
    } else {
        double cu = g.u(i, 0) - prim[1], cv = g.u(i, 1) - prim[2], cw = g.u(i, 2) - prim[3];
        double c2 = cu * cu + cv * cv + cw * cw;
        out[0] = 0.8 * (1 - Pr) * prim[4] * prim[4] / prim[0] * (cu * qf[0] + cv * qf[1] + cw * qf[2]) *
                 (2 * prim[4] * c2 - 5) * H[0];
    }
}
// get_τ (src/Gas/Model.jl:14)
inline double get_tau(const Model& m, const double* prim) {
    return m.prm.mu_ref * 2.0 * std::pow(prim[m.dim + 1], 1 - m.prm.omega) / prim[0];
}
inline double sgn(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0); }
// minmod (Flux/Slope.jl:20-24)
inline double minmod(double a, double b) { return 0.5 * (sgn(a) + sgn(b)) * std::min(std::fabs(a), std::fabs(b)); }

// ------------------------------------------------------------------ slope -------
// diff_vs! / diff_vs_transverse! (Flux/Slope.jl:29-64, 278-332): merge walk of two
// depth-first grids; dm == nullptr selects the plain difference.
void diff_vs(Model& m, const Data& me, const Data& n, double dsL, const double* dm, std::vector<double>& sL) {
    const Grid& g = m.grid_of(me);
    const Grid& gn = m.grid_of(n);
    double* df = m.df(me);
    double* dfn = m.df(n);
    double* sdfn = m.sdfp(n);
    int D = m.dim, NDF = m.ndf, nv = g.nv, nvn = gn.nv;
    auto proj = [&](int j, int k) {
        double p = Model::F(dfn, nvn, j, k);
        if (dm)
            for (int t = 0; t < D; ++t) p += dm[t] * Model::S(sdfn, nvn, NDF, j, k, t);
        return p;
    };
    int index = 0;
    double flag = 0.0;
    for (int i = 0; i < nv; ++i) {
        int li = g.level[i];
        int ln = gn.level[index];
        if (li == ln) {
            for (int k = 0; k < NDF; ++k) sL[(size_t)k * nv + i] += (Model::F(df, nv, i, k) - proj(index, k)) / dsL;
            index += 1;
        } else if (li < ln) {
            while (flag != 1.0) {
                int lj = gn.level[index];
                double sc = std::ldexp(1.0, D * (lj - li));
                for (int k = 0; k < NDF; ++k)
                    sL[(size_t)k * nv + i] += (Model::F(df, nv, i, k) - proj(index, k)) / sc / dsL;
                flag += 1.0 / sc;
                index += 1;
            }
            flag = 0.0;
        } else {
            for (int k = 0; k < NDF; ++k) sL[(size_t)k * nv + i] += (Model::F(df, nv, i, k) - proj(index, k)) / dsL;
            flag += 1.0 / std::ldexp(1.0, D * (li - ln));
            if (flag == 1.0) { index += 1; flag = 0.0; }
        }
    }
}

// _ps_has_transverse_offset (Slope.jl:177-199)
bool has_transverse_offset(Model& m, int c, int k) {
    int D = m.dim, dir = k / 2;
    int n = m.nbr_count(c, k);
    if (n == 0) return false;
    const int32_t* lst = m.nbr_begin(c, k);
    const double* pm = m.t->cell_midpoint + (size_t)c * D;
    for (int t = 0; t < D; ++t) {
        if (t == dir) continue;
        double avg = 0.0;
        for (int j = 0; j < n; ++j) avg += m.mid(m.ref(lst[j]))[t];
        avg /= n;
        if (avg != pm[t]) return true;
    }
    return false;
}

// Sum of diffs over one neighbour list, averaged (update_slope_bound_vs!, inner halves).
void side_slope(Model& m, int c, int k, double ds, bool project, std::vector<double>& s) {
    int D = m.dim, dir = k / 2;
    Data me{1, c};
    const Grid& g = m.grid_of(me);
    std::fill(s.begin(), s.begin() + (size_t)g.nv * m.ndf, 0.0);
    int n = m.nbr_count(c, k);
    const int32_t* lst = m.nbr_begin(c, k);
    const double* pm = m.t->cell_midpoint + (size_t)c * D;
    double dm[3];
    for (int j = 0; j < n; ++j) {
        Data nd = m.ref(lst[j]);
        if (project) {
            const double* nm = m.mid(nd);
            for (int t = 0; t < D; ++t) dm[t] = (t == dir) ? 0.0 : (pm[t] - nm[t]);
            diff_vs(m, me, nd, ds, dm, s);
        } else {
            diff_vs(m, me, nd, ds, nullptr, s);
        }
    }
    for (size_t a = 0; a < (size_t)g.nv * m.ndf; ++a) s[a] /= n;
}

void write_sdf_one(Model& m, int c, int dir, const std::vector<double>& s) {
    Data me{1, c};
    int nv = m.grid_of(me).nv;
    double* sp = m.sdfp(me);
    for (int k = 0; k < m.ndf; ++k)
        for (int i = 0; i < nv; ++i) Model::S(sp, nv, m.ndf, i, k, dir) = s[(size_t)k * nv + i];
}
void write_sdf_minmod(Model& m, int c, int dir, const std::vector<double>& a, const std::vector<double>& b) {
    Data me{1, c};
    int nv = m.grid_of(me).nv;
    double* sp = m.sdfp(me);
    for (int k = 0; k < m.ndf; ++k)
        for (int i = 0; i < nv; ++i)
            Model::S(sp, nv, m.ndf, i, k, dir) = minmod(a[(size_t)k * nv + i], b[(size_t)k * nv + i]);
}

// The neighbour-state dispatcher update_slope!(Val(sL), Val(sR), ...) (Slope.jl:458-771).
void slope_dispatch(Model& m, int c, int dir, std::vector<double>& sL, std::vector<double>& sR) {
    int kL = 2 * dir, kR = 2 * dir + 1;
    int stL = m.nbr_state(c, kL), stR = m.nbr_state(c, kR);
    const double* pm = m.t->cell_midpoint + (size_t)c * m.dim;
    double ds = m.t->cell_ds[(size_t)c * m.dim + dir];
    int half = 1 << (m.dim - 1);
    auto isN = [&](int s) { return s == half; };
    auto first = [&](int k) { return m.ref(m.nbr_begin(c, k)[0]); };
    if (stL == 1 && stR == 1) {
        bool Ls = m.bound_enc(first(kL)) < 0, Rs = m.bound_enc(first(kR)) < 0;
        if (Ls && Rs) {
            Data me{1, c};
            int nv = m.grid_of(me).nv;
            double* sp = m.sdfp(me);
            for (int k = 0; k < m.ndf; ++k)
                for (int i = 0; i < nv; ++i) Model::S(sp, nv, m.ndf, i, k, dir) = 0.0;
        } else if (Ls) {
            side_slope(m, c, kR, pm[dir] - m.mid(first(kR))[dir], false, sL);
            write_sdf_one(m, c, dir, sL);
        } else if (Rs) {
            side_slope(m, c, kL, pm[dir] - m.mid(first(kL))[dir], false, sL);
            write_sdf_one(m, c, dir, sL);
        } else {
            side_slope(m, c, kL, ds, false, sL);
            side_slope(m, c, kR, -ds, false, sR);
            write_sdf_minmod(m, c, dir, sL, sR);
        }
        return;
    }
    if (stL == 0 || stR == 0) {
        if (stL == 0 && stR == 0) { g_err = "cell with domain boundaries on both sides"; throw 1; }
        int k = stL == 0 ? kR : kL;
        side_slope(m, c, k, pm[dir] - m.mid(first(k))[dir], false, sL);
        write_sdf_one(m, c, dir, sL);
        return;
    }
    auto fac = [&](int s, bool left) {
        double v = s == 1 ? 1.0 : (isN(s) ? 0.75 : 1.5);
        return left ? v * ds : -v * ds;
    };
    side_slope(m, c, kL, fac(stL, true), false, sL);
    side_slope(m, c, kR, fac(stR, false), false, sR);
    write_sdf_minmod(m, c, dir, sL, sR);
}

// update_slope_transverse_level! step (2) for one direction (Slope.jl:908-941).
void slope_transverse(Model& m, int c, int dir, std::vector<double>& sL, std::vector<double>& sR) {
    int kL = 2 * dir, kR = 2 * dir + 1;
    int stL = m.nbr_state(c, kL), stR = m.nbr_state(c, kR);
    const double* pm = m.t->cell_midpoint + (size_t)c * m.dim;
    auto first = [&](int k) { return m.ref(m.nbr_begin(c, k)[0]); };
    if (stL != 0 && stR != 0) {
        if (!(stL == -1 || stR == -1)) return;
        double dsL = pm[dir] - m.mid(first(kL))[dir];
        double dsR = pm[dir] - m.mid(first(kR))[dir];
        bool projL = has_transverse_offset(m, c, kL);
        bool projR = has_transverse_offset(m, c, kR);
        side_slope(m, c, kL, dsL, projL, sL);
        side_slope(m, c, kR, dsR, projR, sR);
        write_sdf_minmod(m, c, dir, sL, sR);
        if (m.bound_enc(first(kL)) < 0) {
            side_slope(m, c, kR, dsR, true, sL);
            write_sdf_one(m, c, dir, sL);
        } else if (m.bound_enc(first(kR)) < 0) {
            side_slope(m, c, kL, dsL, true, sL);
            write_sdf_one(m, c, dir, sL);
        }
    } else if (stR == 0 && stL == -1) {
        if (m.bound_enc(first(kL)) < 0) return;
        side_slope(m, c, kL, pm[dir] - m.mid(first(kL))[dir], true, sL);
        write_sdf_one(m, c, dir, sL);
    } else if (stL == 0 && stR == -1) {
        if (m.bound_enc(first(kR)) < 0) return;
        side_slope(m, c, kR, pm[dir] - m.mid(first(kR))[dir], true, sL);
        write_sdf_one(m, c, dir, sL);
    }
}

// slope! (Slope.jl:1047-1070) without the MPI exchanges and the macro slope sw.
void slope(Model& m) {
    int nc = m.t->n_cells;
    int Lmin = INT32_MAX, Lmax = 0;
    for (int c = 0; c < nc; ++c) {
        if (m.t->cell_bound_enc[c] < 0) continue;
        Lmin = std::min(Lmin, (int)m.t->cell_level[c]);
        Lmax = std::max(Lmax, (int)m.t->cell_level[c]);
    }
    if (Lmin == INT32_MAX) Lmin = 0;
    size_t maxnv = 0;
    for (auto& g : m.grids) maxnv = std::max(maxnv, (size_t)g.nv);
    for (int L = Lmin; L <= Lmax; ++L) {
#pragma omp parallel num_threads(m.nthreads)
        {
            std::vector<double> sL(maxnv * m.ndf), sR(maxnv * m.ndf);
#pragma omp for schedule(dynamic, 16)
            for (int c = 0; c < nc; ++c) {
                if (m.t->cell_bound_enc[c] < 0 || m.t->cell_level[c] != L) continue;
                for (int dir = 0; dir < m.dim; ++dir) {
                    int stL = m.nbr_state(c, 2 * dir), stR = m.nbr_state(c, 2 * dir + 1);
                    if (L != Lmin && (stL == -1 || stR == -1)) continue;
                    slope_dispatch(m, c, dir, sL, sR);
                }
                if (L != Lmin && m.dim > 1)
                    for (int dir = 0; dir < m.dim; ++dir) slope_transverse(m, c, dir, sL, sR);
            }
        }
    }
}

// --------------------------------------------------------------- flux ---------
inline void flux_add(Model& m, double* p, double v) {
    if (m.nthreads > 1) {
#pragma omp atomic
        *p += v;
    } else {
        *p += v;
    }
}

// update_micro_flux!(here, there::PsData, heavi) merge walk (Flux/Flux.jl:151-281).
// here_micro / there_micro are indexed by subset position, column k at [k*n + a].
void update_micro_flux_cells(Model& m, const std::vector<double>& hm, int nh, const std::vector<double>& tm, int nt,
                             int here, int there, const std::vector<char>& heavi, bool there_updated) {
    Data hd{1, here}, td{1, there};
    const Grid& g = m.grid_of(hd);
    const Grid& gn = m.grid_of(td);
    double* flux = m.vsflux.data() + m.foff[here];
    double* flux_n = m.vsflux.data() + m.foff[there];
    int D = m.dim, NDF = m.ndf, nv = g.nv, nvn = gn.nv;
    int index = 0, j = 0, index_n = 0;
    double flag = 0.0;
    auto HM = [&](int a, int k) { return hm[(size_t)k * nh + a]; };
    auto TM = [&](int a, int k) { return tm[(size_t)k * nt + a]; };
    for (int i = 0; i < nv; ++i) {
        int li = g.level[i];
        if (heavi[i]) {
            for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux, nv, i, k), HM(index, k));
            if (li == gn.level[j]) {
                if (there_updated) for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux_n, nvn, j, k), -HM(index, k));
                j += 1;
            } else if (li < gn.level[j]) {
                while (flag != 1.0) {
                    if (there_updated) for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux_n, nvn, j, k), -HM(index, k));
                    flag += 1.0 / std::ldexp(1.0, D * (gn.level[j] - li));
                    j += 1;
                }
                flag = 0.0;
            } else {
                double sc = std::ldexp(1.0, D * (li - gn.level[j]));
                if (there_updated) for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux_n, nvn, j, k), -(HM(index, k) / sc));
                flag += 1.0 / sc;
                if (flag == 1.0) { j += 1; flag = 0.0; }
            }
            index += 1;
        } else {
            if (li == gn.level[j]) {
                for (int k = 0; k < NDF; ++k) {
                    if (there_updated) flux_add(m, &Model::F(flux_n, nvn, j, k), -TM(index_n, k));
                    flux_add(m, &Model::F(flux, nv, i, k), TM(index_n, k));
                }
                j += 1; index_n += 1;
            } else if (li < gn.level[j]) {
                while (flag != 1.0) {
                    double sc = std::ldexp(1.0, D * (gn.level[j] - li));
                    for (int k = 0; k < NDF; ++k) {
                        if (there_updated) flux_add(m, &Model::F(flux_n, nvn, j, k), -TM(index_n, k));
                        flux_add(m, &Model::F(flux, nv, i, k), TM(index_n, k) / sc);
                    }
                    flag += 1.0 / sc;
                    j += 1; index_n += 1;
                }
                flag = 0.0;
            } else {
                for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux, nv, i, k), TM(index_n, k));
                flag += 1.0 / std::ldexp(1.0, D * (li - gn.level[j]));
                if (flag == 1.0) {
                    if (there_updated) for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux_n, nvn, j, k), -TM(index_n, k));
                    j += 1; index_n += 1; flag = 0.0;
                }
            }
        }
    }
}

// positivity_preserving_reconstruct (Flux/CAIDVM.jl:127-142) for subset element (i, k)
inline double pp_recon(const Model& m, double fik, const double* sdfp, int nv, int i, int k, const double* ds, const double* dx) {
    double s_abs = 0, s_dx = 0;
    for (int d = 0; d < m.dim; ++d) s_abs += ds[d] * std::fabs(Model::S(const_cast<double*>(sdfp), nv, m.ndf, i, k, d));
    for (int d = 0; d < m.dim; ++d) s_dx += dx[d] * Model::S(const_cast<double*>(sdfp), nv, m.ndf, i, k, d);
    return fik + std::min(std::fabs((fik - JL_EPS) / (0.5 * s_abs + EPS_REF)), 1.0) * s_dx;
}
inline double plain_recon(const Model& m, double fik, const double* sdfp, int nv, int i, int k, const double* dx) {
    double s = 0;
    for (int d = 0; d < m.dim; ++d) s += dx[d] * Model::S(const_cast<double*>(sdfp), nv, m.ndf, i, k, d);
    return fik + s;
}

// One inner (sub-)face: make_face_vs + calc_flux(CAIDVM|DVM) + update_flux! (Flux.jl:28-59,94-111,362-401;
// CAIDVM.jl:99-121; DVM.jl:79-99).
void inner_face(Model& m, int fi) {
    const kg_topology* t = m.t;
    int D = m.dim, NDF = m.ndf, dir = t->face_dir[fi];
    double rot = t->face_rot[fi], area = t->face_area[fi];
    const double* fmid = t->face_midpoint + (size_t)fi * D;
    const double* tmid = t->face_there_midpoint + (size_t)fi * D;
    int here = t->face_here[fi];
    Data hd{1, here};
    Data td = m.ref(t->face_there[fi]);
    const Grid& g = m.grid_of(hd);
    const Grid& gn = m.grid_of(td);
    double* hf = m.df(hd);
    double* hs = m.sdfp(hd);
    double* tf = m.df(td);
    double* ts = m.sdfp(td);
    const double* hmid = t->cell_midpoint + (size_t)here * D;
    const double* hds = t->cell_ds + (size_t)here * D;
    const double* tds = m.ds(td);
    bool there_solid = m.bound_enc(td) < 0;
    double dt = m.dt;
    std::vector<char> heavi(g.nv);
    std::vector<int> hsel, tsel;
    for (int i = 0; i < g.nv; ++i) { heavi[i] = (rot * g.u(i, dir) <= 0.0); if (heavi[i]) hsel.push_back(i); }
    for (int i = 0; i < gn.nv; ++i) if (rot * gn.u(i, dir) > 0.0) tsel.push_back(i);
    int nh = (int)hsel.size(), nt = (int)tsel.size();
    std::vector<double> hm((size_t)NDF * nh), tm((size_t)NDF * nt);
    double dx[3];
    for (int a = 0; a < nh; ++a) {
        int i = hsel[a];
        for (int d = 0; d < D; ++d) dx[d] = fmid[d] - g.u(i, d) * dt - hmid[d];
        double vn = g.u(i, dir);
        for (int k = 0; k < NDF; ++k) {
            double fik = Model::F(hf, g.nv, i, k);
            double r = there_solid ? plain_recon(m, fik, hs, g.nv, i, k, dx) : pp_recon(m, fik, hs, g.nv, i, k, hds, dx);
            hm[(size_t)k * nh + a] = r * vn;
        }
    }
    for (int a = 0; a < nt; ++a) {
        int i = tsel[a];
        for (int d = 0; d < D; ++d) dx[d] = fmid[d] - gn.u(i, d) * dt - tmid[d];
        double vn = gn.u(i, dir);
        for (int k = 0; k < NDF; ++k) {
            double fik = Model::F(tf, gn.nv, i, k);
            double r;
            if (there_solid)
                r = (m.prm.flux == KG_FLUX_CAIDVM) ? fik : plain_recon(m, fik, ts, gn.nv, i, k, dx);
            else
                r = pp_recon(m, fik, ts, gn.nv, i, k, tds, dx);
            tm[(size_t)k * nt + a] = r * vn;
        }
    }
    bool there_updated = (td.kind == 1) && !there_solid;
    if (m.prm.flux == KG_FLUX_CAIDVM) {
        double fw1[5], fw2[5];
        moments_subset(m, g, hsel, hm, fw1);
        moments_subset(m, gn, tsel, tm, fw2);
        for (int e = 0; e < m.nw(); ++e) {
            double v = (fw1[e] + fw2[e]) * area;
            flux_add(m, &m.wflux[(size_t)here * m.nw() + e], v);
            if (there_updated) flux_add(m, &m.wflux[(size_t)td.idx * m.nw() + e], -v);
        }
    }
    for (auto& v : hm) v *= area;
    for (auto& v : tm) v *= area;
    if (td.kind == 2) {
        // update_micro_flux!(…, ::SolidNeighbor, heavi) (Flux.jl:140-146): same grid
        double* flux = m.vsflux.data() + m.foff[here];
        int a = 0, b = 0;
        for (int i = 0; i < g.nv; ++i) {
            if (heavi[i]) { for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux, g.nv, i, k), hm[(size_t)k * nh + a]); ++a; }
            else { for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux, g.nv, i, k), tm[(size_t)k * nt + b]); ++b; }
        }
    } else {
        update_micro_flux_cells(m, hm, nh, tm, nt, here, td.idx, heavi, there_updated);
    }
}

// DomainFace: make_face_vs + calc_domain_flux + update_domain_flux! (Flux.jl:19-24,64-83,349-358;
// CAIDVM.jl:4-94; DVM.jl:1-77)
void domain_face(Model& m, int fi) {
    const kg_topology* t = m.t;
    int D = m.dim, NDF = m.ndf, dir = t->face_dir[fi];
    double rot = t->face_rot[fi], area = t->face_area[fi];
    const double* fmid = t->face_midpoint + (size_t)fi * D;
    int c = t->face_here[fi];
    Data cd{1, c};
    const Grid& g = m.grid_of(cd);
    int nv = g.nv;
    double* cf = m.df(cd);
    double* cs = m.sdfp(cd);
    const double* cmid = t->cell_midpoint + (size_t)c * D;
    double dt = m.dt;
    int kind = t->face_bc_kind[fi];
    std::vector<char> heavi(nv);
    std::vector<int> hsel, tsel;
    for (int i = 0; i < nv; ++i) { heavi[i] = (rot * g.u(i, dir) <= 0.0); if (heavi[i]) hsel.push_back(i); else tsel.push_back(i); }
    int nh = (int)hsel.size(), nt = (int)tsel.size();
    std::vector<double> hm((size_t)NDF * nh), tm((size_t)NDF * nt);
    double dx[3];
    double bc[5];
    for (int e = 0; e < D + 2; ++e) bc[e] = t->face_bc[(size_t)fi * (D + 2) + e];
    if (kind == KG_BC_MAXWELL || kind == KG_BC_INFLOW) {
        if (kind == KG_BC_MAXWELL && m.prm.flux == KG_FLUX_DVM) {
            g_err = "DVM Maxwellian domain flux is undefined in the reference (DVM.jl:3,12)";
            throw 1;
        }
        std::vector<double> df((size_t)NDF * nh);
        for (int a = 0; a < nh; ++a) {
            int i = hsel[a];
            for (int d = 0; d < D; ++d) dx[d] = fmid[d] - g.u(i, d) * dt - cmid[d];
            for (int k = 0; k < NDF; ++k) df[(size_t)k * nh + a] = plain_recon(m, Model::F(cf, nv, i, k), cs, nv, i, k, dx);
        }
        if (kind == KG_BC_MAXWELL) {
            // calc_ρw (Theory/Math.jl:251-282)
            double SF = 0, SG = 0;
            for (int a = 0; a < nh; ++a) { int i = hsel[a]; SF += g.weight[i] * g.u(i, dir) * df[a]; }
            for (int a = 0; a < nt; ++a) {
                int i = tsel[a];
                double c2 = 0;
                for (int d = 0; d < D; ++d) c2 += (g.u(i, d) - bc[1 + d]) * (g.u(i, d) - bc[1 + d]);
                SG += g.weight[i] * g.u(i, dir) * std::exp(-bc[D + 1] * c2);
            }
            SG *= (D == 2) ? bc[3] / PI : std::pow(bc[4] / PI, 1.5);
            bc[0] = -SF / SG;
        }
        double M[2];
        for (int a = 0; a < nh; ++a)
            for (int k = 0; k < NDF; ++k) hm[(size_t)k * nh + a] = df[(size_t)k * nh + a] * g.u(hsel[a], dir);
        for (int a = 0; a < nt; ++a) {
            maxwell(m, g, tsel[a], bc, M);
            for (int k = 0; k < NDF; ++k) tm[(size_t)k * nt + a] = M[k] * g.u(tsel[a], dir);
        }
    } else if (kind == KG_BC_OUTFLOW) {
        for (int a = 0; a < nh; ++a)
            for (int k = 0; k < NDF; ++k) hm[(size_t)k * nh + a] = Model::F(cf, nv, hsel[a], k) * g.u(hsel[a], dir);
        for (int a = 0; a < nt; ++a)
            for (int k = 0; k < NDF; ++k) tm[(size_t)k * nt + a] = Model::F(cf, nv, tsel[a], k) * g.u(tsel[a], dir);
    } else if (kind == KG_BC_INTERP) {
        if (D != 2) { g_err = "InterpolatedOutflow is 2D only in the reference"; throw 1; }
        double tpm[3];
        for (int d = 0; d < D; ++d) tpm[d] = 2.0 * fmid[d] - cmid[d];
        for (int a = 0; a < nh; ++a) {
            int i = hsel[a];
            for (int d = 0; d < D; ++d) dx[d] = fmid[d] - g.u(i, d) * dt - cmid[d];
            for (int k = 0; k < NDF; ++k) hm[(size_t)k * nh + a] = plain_recon(m, Model::F(cf, nv, i, k), cs, nv, i, k, dx) * g.u(i, dir);
        }
        for (int a = 0; a < nt; ++a) {
            int i = tsel[a];
            for (int d = 0; d < D; ++d) dx[d] = fmid[d] - g.u(i, d) * dt - tpm[d];
            for (int k = 0; k < NDF; ++k) {
                double tdf = Model::F(cf, nv, i, k) + (tpm[dir] - cmid[dir]) * Model::S(cs, nv, NDF, i, k, dir);
                tm[(size_t)k * nt + a] = plain_recon(m, tdf, cs, nv, i, k, dx) * g.u(i, dir);
            }
        }
    } else {
        g_err = "unknown domain boundary kind";
        throw 1;
    }
    if (m.prm.flux == KG_FLUX_CAIDVM) {
        double fw1[5], fw2[5];
        moments_subset(m, g, hsel, hm, fw1);
        moments_subset(m, g, tsel, tm, fw2);
        for (int e = 0; e < m.nw(); ++e) flux_add(m, &m.wflux[(size_t)c * m.nw() + e], area * (fw1[e] + fw2[e]));
    }
    double* flux = m.vsflux.data() + m.foff[c];
    for (int a = 0; a < nh; ++a)
        for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux, nv, hsel[a], k), area * hm[(size_t)k * nh + a]);
    for (int a = 0; a < nt; ++a)
        for (int k = 0; k < NDF; ++k) flux_add(m, &Model::F(flux, nv, tsel[a], k), area * tm[(size_t)k * nt + a]);
}

// fluid neighbours of a cell: first entry of each faceid list that is a PsData with
// bound_enc >= 0 (Immersed_boundary.jl:143-144, 368-372)
std::vector<int> fluid_neighbours(Model& m, int c) {
    std::vector<int> out;
    for (int k = 0; k < 2 * m.dim; ++k) {
        int32_t r = m.nbr_begin(c, k)[0];
        if (r >= 0 && m.t->cell_bound_enc[r] >= 0) out.push_back(r);
    }
    return out;
}

// vs_extrapolate! (Immersed_boundary.jl:98-121): dft += weight * merge(df + sdf.dx)
void vs_extrapolate(Model& m, int src, double* dft, const Grid& gt, const double* dx, const std::vector<double>& wi) {
    Data sd{1, src};
    const Grid& g = m.grid_of(sd);
    double* df = m.df(sd);
    double* sdf = m.sdfp(sd);
    int D = m.dim, NDF = m.ndf;
    auto val = [&](int j, int k) {
        double s = 0;
        for (int d = 0; d < D; ++d) s += Model::S(sdf, g.nv, NDF, j, k, d) * dx[d];
        return Model::F(df, g.nv, j, k) + s;
    };
    int j = 0;
    double flag = 0.0;
    for (int i = 0; i < gt.nv; ++i) {
        int lt = gt.level[i];
        if (lt == g.level[j]) {
            for (int k = 0; k < NDF; ++k) Model::F(dft, gt.nv, i, k) += val(j, k) * wi[i];
            j += 1;
        } else if (lt < g.level[j]) {
            while (flag != 1.0) {
                double sc = std::ldexp(1.0, D * (g.level[j] - lt));
                for (int k = 0; k < NDF; ++k) Model::F(dft, gt.nv, i, k) += val(j, k) / sc * wi[i];
                flag += 1.0 / sc;
                j += 1;
            }
            flag = 0.0;
        } else {
            for (int k = 0; k < NDF; ++k) Model::F(dft, gt.nv, i, k) += val(j, k) * wi[i];
            flag += 1.0 / std::ldexp(1.0, D * (lt - g.level[j]));
            if (flag == 1.0) { j += 1; flag = 0.0; }
        }
    }
}

// directional weights max(0, u.l/|u|)^2 normalised over the donor set
// (Immersed_boundary.jl:124-135, 379-390)
void extrapolate_from(Model& m, const std::vector<int>& cells, const double* target_point, double* dft, const Grid& gt) {
    int D = m.dim, n = (int)cells.size();
    std::vector<double> W((size_t)gt.nv * n), wsum(gt.nv, 0.0), wi(gt.nv);
    for (int a = 0; a < n; ++a) {
        const double* cm = m.t->cell_midpoint + (size_t)cells[a] * D;
        double l[3], nl = 0;
        for (int d = 0; d < D; ++d) { l[d] = target_point[d] - cm[d]; nl += l[d] * l[d]; }
        nl = std::sqrt(nl);
        for (int d = 0; d < D; ++d) l[d] /= nl;
        for (int i = 0; i < gt.nv; ++i) {
            double ul = 0, uu = 0;
            for (int d = 0; d < D; ++d) { ul += gt.u(i, d) * l[d]; uu += gt.u(i, d) * gt.u(i, d); }
            double v = std::max(0.0, ul / std::sqrt(uu));
            W[(size_t)i * n + a] = v * v;
        }
    }
    for (int i = 0; i < gt.nv; ++i) {
        double s = 0;
        for (int a = 0; a < n; ++a) s += W[(size_t)i * n + a];
        wsum[i] = s;
    }
    for (int a = 0; a < n; ++a) {
        for (int i = 0; i < gt.nv; ++i) wi[i] = wsum[i] == 0.0 ? 1.0 / n : W[(size_t)i * n + a] / wsum[i];
        const double* cm = m.t->cell_midpoint + (size_t)cells[a] * D;
        double dx[3];
        for (int d = 0; d < D; ++d) dx[d] = target_point[d] - cm[d];
        vs_extrapolate(m, cells[a], dft, gt, dx, wi);
    }
}

// update_solid_cell! (Immersed_boundary.jl:122-146, 207-213)
void update_solid_cells(Model& m) {
    int nc = m.t->n_cells, D = m.dim;
#pragma omp parallel for num_threads(m.nthreads) schedule(dynamic, 4)
    for (int c = 0; c < nc; ++c) {
        if (m.t->cell_bound_enc[c] >= 0) continue;
        Data cd{1, c};
        const Grid& g = m.grid_of(cd);
        double* df = m.df(cd);
        std::fill(df, df + (size_t)g.nv * m.ndf, 0.0);
        std::vector<int> fl = fluid_neighbours(m, c);
        extrapolate_from(m, fl, m.t->cell_midpoint + (size_t)c * D, df, g);
        double* w = m.w + (size_t)c * m.nw();
        calc_w0(m, g, df, w);
        get_prim(m, w, m.prim + (size_t)c * m.nw());
    }
}

// update_solid_neighbor! (Immersed_boundary.jl:436-483)
void update_walls(Model& m) {
    const kg_topology* t = m.t;
    int D = m.dim, NDF = m.ndf;
#pragma omp parallel for num_threads(m.nthreads) schedule(dynamic, 1)
    for (int w = 0; w < t->n_walls; ++w) {
        int c = t->wall_donor[w], s = t->wall_solid[w];
        int dir = t->wall_faceid[w] / 2;
        Data cd{1, c}, sd{1, s}, wd{2, w};
        const Grid& g = m.grid_of(cd);
        const Grid& gs = m.grid_of(sd);
        int nv = g.nv;
        const double* aux = t->wall_aux_point + (size_t)w * D;
        const double* nrm = t->wall_normal + (size_t)w * D;
        const double* cm = t->cell_midpoint + (size_t)c * D;
        const double* sm = t->cell_midpoint + (size_t)s * D;
        double* cf = m.df(cd);
        double* sf = m.df(sd);
        std::vector<double> vn(nv), theta(nv);
        for (int i = 0; i < nv; ++i) {
            double v = 0;
            for (int d = 0; d < D; ++d) v += g.u(i, d) * nrm[d];
            vn[i] = v;
            theta[i] = v >= 0 ? 1.0 : 0.0;  // heaviside (Theory/Math.jl:4)
        }
        double ib_point[3];
        for (int d = 0; d < D; ++d) ib_point[d] = aux[d] + cm[d] - sm[d];
        // image_df: fluid neighbours of the donor, then the donor itself
        std::vector<double> ib((size_t)nv * NDF, 0.0);
        std::vector<int> fl = fluid_neighbours(m, c);
        fl.push_back(c);
        extrapolate_from(m, fl, ib_point, ib.data(), g);
        // boundary_slope! (Immersed_boundary.jl:396-435)
        double dxf = ib_point[dir] - cm[dir];
        double dxs = cm[dir] - sm[dir];
        std::vector<double> sL((size_t)nv * NDF, 0.0);
        {
            int index = 0;
            double flag = 0.0;
            for (int i = 0; i < nv; ++i) {
                int li = g.level[i];
                if (li == gs.level[index]) {
                    for (int k = 0; k < NDF; ++k) sL[(size_t)k * nv + i] = (Model::F(cf, nv, i, k) - Model::F(sf, gs.nv, index, k)) / dxs;
                    index += 1;
                } else if (li < gs.level[index]) {
                    while (flag != 1.0) {
                        double sc = std::ldexp(1.0, D * (gs.level[index] - li));
                        for (int k = 0; k < NDF; ++k)
                            sL[(size_t)k * nv + i] += (Model::F(cf, nv, i, k) - Model::F(sf, gs.nv, index, k)) / sc / dxs;
                        flag += 1.0 / sc;
                        index += 1;
                    }
                    flag = 0.0;
                } else {
                    for (int k = 0; k < NDF; ++k) sL[(size_t)k * nv + i] += (Model::F(cf, nv, i, k) - Model::F(sf, gs.nv, index, k)) / dxs;
                    flag += 1.0 / std::ldexp(1.0, D * (li - gs.level[index]));
                    if (flag == 1.0) { index += 1; flag = 0.0; }
                }
            }
        }
        double dxL = aux[dir] - ib_point[dir];
        double* wsdf = m.sdfp(wd);
        std::vector<double> aux_df((size_t)nv * NDF);
        for (int k = 0; k < NDF; ++k)
            for (int i = 0; i < nv; ++i) {
                double ss = minmod(sL[(size_t)k * nv + i], (ib[(size_t)k * nv + i] - Model::F(cf, nv, i, k)) / dxf);
                ss = std::min(std::fabs((ib[(size_t)k * nv + i] - JL_EPS) / (ss * dxL + JL_EPS)), 1.0) * ss;
                Model::S(wsdf, nv, NDF, i, k, dir) = ss;
                aux_df[(size_t)k * nv + i] = ib[(size_t)k * nv + i] + ss * dxL;
            }
        // cut cells (cvc_gas_correction!, cvc_Mu, cvc_density, cvc_correction!; :332-366)
        int c0 = t->wall_cut_off[w], c1 = t->wall_cut_off[w + 1], ncut = c1 - c0;
        std::vector<double> cw(g.weight, g.weight + nv);
        for (int a = 0; a < ncut; ++a) cw[t->wall_cut_index[c0 + a]] = 0.0;
        std::vector<double> gas_dfs((size_t)ncut * NDF);
        for (int a = 0; a < ncut; ++a)
            for (int k = 0; k < NDF; ++k) gas_dfs[(size_t)k * ncut + a] = aux_df[(size_t)k * nv + t->wall_cut_index[c0 + a]];
        double ap[5];
        for (int e = 0; e < D + 2; ++e) ap[e] = t->wall_bc[(size_t)w * (D + 2) + e];
        ap[0] = 1.0;
        std::vector<double> M((size_t)nv * NDF);
        double mm[2];
        for (int i = 0; i < nv; ++i) {
            maxwell(m, g, i, ap, mm);
            for (int k = 0; k < NDF; ++k) M[(size_t)k * nv + i] = mm[k];
        }
        double MuL = 0, MuR = 0;
        for (int i = 0; i < nv; ++i) MuL += cw[i] * vn[i] * M[i] * (1.0 - theta[i]);
        for (int i = 0; i < nv; ++i) MuR += cw[i] * vn[i] * M[i] * theta[i];
        for (int a = 0; a < ncut; ++a) {
            int i = t->wall_cut_index[c0 + a];
            MuL += t->wall_cut_gas_w[c0 + a] * vn[i] * M[i];
            MuR += t->wall_cut_solid_w[c0 + a] * vn[i] * M[i];
        }
        (void)MuL;
        double SF = 0;
        for (int i = 0; i < nv; ++i) SF += cw[i] * vn[i] * aux_df[i] * (1.0 - theta[i]);
        for (int a = 0; a < ncut; ++a) {
            int i = t->wall_cut_index[c0 + a];
            SF += t->wall_cut_gas_w[c0 + a] * vn[i] * gas_dfs[a];
        }
        double rho_w = -SF / MuR;
        for (auto& v : M) v *= rho_w;
        for (int i = 0; i < nv; ++i)
            if (theta[i] == 1.0)
                for (int k = 0; k < NDF; ++k) aux_df[(size_t)k * nv + i] = M[(size_t)k * nv + i];
        for (int a = 0; a < ncut; ++a) {
            int i = t->wall_cut_index[c0 + a];
            double gw = t->wall_cut_gas_w[c0 + a], sw = t->wall_cut_solid_w[c0 + a];
            for (int k = 0; k < NDF; ++k)
                aux_df[(size_t)k * nv + i] = (gw * gas_dfs[(size_t)k * ncut + a] + sw * M[(size_t)k * nv + i]) / (gw + sw);
        }
        double* wf = m.df(wd);
        std::copy(aux_df.begin(), aux_df.end(), wf);
    }
}

void flux(Model& m) {
    const kg_topology* t = m.t;
    update_solid_cells(m);
    auto is_ib = [&](int fi) { return t->face_kind[fi] == KG_FACE_INNER && t->face_there[fi] < 0; };
#pragma omp parallel for num_threads(m.nthreads) schedule(dynamic, 8)
    for (int fi = 0; fi < t->n_faces; ++fi) {
        if (is_ib(fi)) continue;
        if (t->face_kind[fi] == KG_FACE_DOMAIN) domain_face(m, fi);
        else inner_face(m, fi);
    }
    update_walls(m);
#pragma omp parallel for num_threads(m.nthreads) schedule(dynamic, 8)
    for (int fi = 0; fi < t->n_faces; ++fi)
        if (is_ib(fi)) inner_face(m, fi);
}

// ---------------------------------------------------------- I-projection --------
// solve_I_projection (Theory/I-projection.jl:55-141): Newton iterations on the dual equation
// G(λ) = Σ_k ω_k f_k exp(λ·ψ_k) ψ_k - W = 0, ψ_k = (1, ξ_k, |ξ_k|²/2), from λ = 0, with the
// reference's negative-value shave of f (in place), its stall test and its Armijo
// backtracking on the dual objective Φ(λ) = Σ_k ω_k f_k exp(λ·ψ_k) - λ·W.  The symmetric
// Newton system is solved by Gaussian elimination with partial pivoting (the reference calls
// a symmetric factorisation; the two agree to rounding).  Returns the iterations taken.
static void iproj_psi(int D, const double* mid, int nv, int k, double* psi) {
    psi[0] = 1.0;
    double s = 0.0;
    for (int d = 0; d < D; ++d) {
        const double x = mid[(size_t)d * nv + k];
        psi[1 + d] = x;
        s += x * x;
    }
    psi[D + 1] = s / 2;
}
static double iproj_dual(int D, const double* mid, const double* wt, const double* f, int nv, const double* W,
                         const double* lam) {
    const int M = D + 2;
    double acc = 0.0, psi[5];
    for (int k = 0; k < nv; ++k) {
        iproj_psi(D, mid, nv, k, psi);
        double dot = 0.0;
        for (int i = 0; i < M; ++i) dot += lam[i] * psi[i];
        acc += wt[k] * f[k] * std::exp(dot);
    }
    double lw = 0.0;
    for (int i = 0; i < M; ++i) lw += lam[i] * W[i];
    return acc - lw;
}
// x = A⁻¹ b for a small dense system (n ≤ 5), partial pivoting
static void small_solve(int n, double (*A)[5], double* b, double* x) {
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[r][c]) > std::fabs(A[p][c])) p = r;
        if (p != c) {
            for (int j = 0; j < n; ++j) std::swap(A[c][j], A[p][j]);
            std::swap(b[c], b[p]);
        }
        for (int r = c + 1; r < n; ++r) {
            const double l = A[r][c] / A[c][c];
            for (int j = c; j < n; ++j) A[r][j] -= l * A[c][j];
            b[r] -= l * b[c];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = b[r];
        for (int j = r + 1; j < n; ++j) s -= A[r][j] * x[j];
        x[r] = s / A[r][r];
    }
}
int solve_iprojection(int D, const double* mid, double* f, const double* W, const double* wt, int nv, double* lam) {
    const int M = D + 2, maxiter = 10;
    double wn = 0.0;
    for (int i = 0; i < M; ++i) wn += W[i] * W[i];
    const double tol_eff = 1e-10 * std::max(1.0, std::sqrt(wn));
    for (int i = 0; i < M; ++i) lam[i] = 0.0;
    // shave negative distribution
    double fmn = INFINITY;
    for (int k = 0; k < nv; ++k) fmn = std::min(fmn, f[k]);
    const double f_min = 1.1 * fmn;
    if (f_min < 0) {
        double fp_min = INFINITY;
        for (int k = 0; k < nv; ++k)
            if (f[k] > 0) fp_min = std::min(fp_min, f[k]);
        if (fp_min < INFINITY) {
            const double d = fp_min - f_min;
            for (int k = 0; k < nv; ++k)
                if (f[k] < 0) f[k] = (f[k] - f_min) / d * fp_min;
        }
    }
    double Gprev = INFINITY;
    int stall = 0, it = 0;
    for (; it < maxiter; ++it) {
        double G[5] = {0, 0, 0, 0, 0}, J[5][5] = {}, psi[5];
        for (int k = 0; k < nv; ++k) {
            iproj_psi(D, mid, nv, k, psi);
            double dot = 0.0;
            for (int i = 0; i < M; ++i) dot += lam[i] * psi[i];
            const double c = wt[k] * f[k] * std::exp(dot);
            for (int i = 0; i < M; ++i) {
                const double ci = c * psi[i];
                G[i] += ci;
                for (int j = i; j < M; ++j) J[i][j] += ci * psi[j];
            }
        }
        double gn = 0.0;
        for (int i = 0; i < M; ++i) { G[i] -= W[i]; gn += G[i] * G[i]; }
        gn = std::sqrt(gn);
        if (gn < tol_eff) return it;
        if (gn > 0.9 * Gprev) {
            if (++stall >= 2) return it;
        } else {
            stall = 0;
        }
        Gprev = gn;
        for (int i = 0; i < M; ++i)
            for (int j = 0; j < i; ++j) J[i][j] = J[j][i];
        double rhs[5], dl[5];
        for (int i = 0; i < M; ++i) rhs[i] = -G[i];
        small_solve(M, J, rhs, dl);
        const double phi0 = iproj_dual(D, mid, wt, f, nv, W, lam);
        double slope = 0.0;
        for (int i = 0; i < M; ++i) slope += G[i] * dl[i];
        double alpha = 1.0, trial[5];
        for (int ls = 0; ls < maxiter; ++ls) {
            for (int i = 0; i < M; ++i) trial[i] = lam[i] + alpha * dl[i];
            if (iproj_dual(D, mid, wt, f, nv, W, trial) <= phi0 + 1e-4 * alpha * slope) break;
            alpha *= 0.5;
        }
        for (int i = 0; i < M; ++i) lam[i] += alpha * dl[i];
    }
    return it;
}
// conserved_I_porjection! (Theory/I-projection.jl:144-158): 2D2F projects df[:,1] onto w with
// the energy of df[:,2] taken out; 3D1F projects df onto w
void conserved_iprojection(int D, int NDF, const double* mid, const double* wt, int nv, double* df, const double* w,
                           double* lam) {
    if (D != 2 && D != 3) return;
    const int M = D + 2;
    double W[5];
    for (int i = 0; i < M; ++i) W[i] = w[i];
    if (NDF == 2) {
        double e = 0.0;
        for (int k = 0; k < nv; ++k) e += wt[k] * df[nv + k];
        W[M - 1] -= e / 2;
    }
    solve_iprojection(D, mid, df, W, wt, nv, lam);
    double psi[5];
    for (int k = 0; k < nv; ++k) {
        iproj_psi(D, mid, nv, k, psi);
        double dot = 0.0;
        for (int i = 0; i < M; ++i) dot += lam[i] * psi[i];
        df[k] *= std::exp(dot);
    }
}

// ------------------------------------------------------------- iterate --------
// iterate!(CAIDVM_Marching) (Theory/Iterate.jl:96-130), iterate!(Euler) (:131-162) and
// iterate!(CIP_Marching) (Theory/I-projection.jl:161-193)
// positivity_preserving_ib! (Boundary/Positivity.jl:1-43) of donor cell c (CIP marching,
// after the macroscopic update): per SolidNeighbor, in face order, the velocities entering
// from the wall (rot u_dir > 0) carry the reconstruction perturbance of update_solid_neighbor!
// -- the record's flux ssdf (x_solid - x_aux) along dir, reconstructed with the record's sdf
// (zero but for its wall-direction slope) from the solid centre to the face -- times u_dir and
// the signed face area.  Their moments, scaled by dt / volume, enter w with the largest
// factor theta <= 1 that keeps the density and the internal energy positive (margin 1e-3),
// and theta times the micro fluxes join the cell's velocity-space flux.
void positivity_ib(Model& m, int c, double volume) {
    const kg_topology* t = m.t;
    const int D = m.dim, NDF = m.ndf, NW = m.nw();
    Data cd{1, c};
    const Grid& g = m.grid_of(cd);
    const int nv = g.nv;
    std::vector<int> walls;
    for (int w = 0; w < t->n_walls; ++w)
        if (t->wall_donor[w] == c) walls.push_back(w);
    std::sort(walls.begin(), walls.end(), [&](int a, int b) { return t->wall_faceid[a] < t->wall_faceid[b]; });
    if (walls.empty()) return;
    const double* cm = t->cell_midpoint + (size_t)c * D;
    const double* ds = t->cell_ds + (size_t)c * D;
    std::vector<double> micros(walls.size() * (size_t)nv * NDF, 0.0);
    double we[5] = {0, 0, 0, 0, 0};
    for (size_t j = 0; j < walls.size(); ++j) {
        const int w = walls[j];
        const int k = t->wall_faceid[w], dir = k / 2;
        const double rot = (k % 2 == 0) ? 1.0 : -1.0;
        double fmid[3] = {0.0, 0.0, 0.0};
        for (int d = 0; d < D; ++d) fmid[d] = cm[d];
        fmid[dir] -= 0.5 * rot * ds[dir];
        const double* sm = t->cell_midpoint + (size_t)t->wall_solid[w] * D;
        const double* aux = t->wall_aux_point + (size_t)w * D;
        double area = rot;
        for (int d = 0; d < D; ++d)
            if (d != dir) area *= ds[d];
        Data wd{2, w};
        double* wsdf = m.sdfp(wd);
        double* mic = micros.data() + j * (size_t)nv * NDF;
        for (int i = 0; i < nv; ++i) {
            const double vn = g.u(i, dir);
            if (!(rot * vn > 0.0)) continue;
            for (int kk = 0; kk < NDF; ++kk) {
                const double ndf = Model::S(wsdf, nv, NDF, i, kk, dir) * (sm[dir] - aux[dir]);
                double dot = 0.0;
                for (int d = 0; d < D; ++d) dot += (fmid[d] - g.u(i, d) * m.dt - sm[d]) * Model::S(wsdf, nv, NDF, i, kk, d);
                mic[(size_t)kk * nv + i] = (ndf + dot) * vn * area;
            }
        }
        double wm[5];
        calc_w0(m, g, mic, wm);
        for (int e = 0; e < NW; ++e) we[e] += wm[e];
    }
    for (int e = 0; e < NW; ++e) we[e] *= m.dt / volume;
    double* wb = m.w + (size_t)c * NW;
    const double delta = 1e-3;
    const double th_rho = we[0] > 0.0 ? 1.0 : std::min(1.0, (1.0 - delta) * wb[0] / (std::fabs(we[0]) + JL_EPS));
    double rub2 = 0.0, rue2 = 0.0, rbe = 0.0;
    for (int d = 0; d < D; ++d) { rub2 += wb[1 + d] * wb[1 + d]; rue2 += we[1 + d] * we[1 + d]; rbe += wb[1 + d] * we[1 + d]; }
    const double eb = wb[D + 1] - rub2 / (2.0 * wb[0]);
    const double ee = we[D + 1] - rbe / wb[0];
    const double gam = rue2 / (2.0 * wb[0]);
    const double th_e = std::min(1.0, 2.0 * (1.0 - delta) * eb / (std::sqrt(ee * ee + 4.0 * gam * (1.0 - delta) * eb) - ee + JL_EPS));
    const double th = std::min(th_rho, th_e);
    for (int e = 0; e < NW; ++e) wb[e] += th * we[e];
    double* vf = m.vsflux.data() + m.foff[c];
    for (size_t j = 0; j < walls.size(); ++j) {
        const double* mic = micros.data() + j * (size_t)nv * NDF;
        for (size_t a = 0; a < (size_t)nv * NDF; ++a) vf[a] += th * mic[a];
    }
}

void iterate(Model& m, int64_t step, double* sum_res, double* sum_avg) {
    const kg_topology* t = m.t;
    int D = m.dim, NDF = m.ndf, NW = m.nw();
    double dt = m.dt;
    bool check = (step % m.prm.st_check_interval) == 0;
    int nc = t->n_cells;
    std::vector<double> res((size_t)nc * NW, 0.0), avg((size_t)nc * NW, 0.0);
#pragma omp parallel for num_threads(m.nthreads) schedule(dynamic, 4)
    for (int c = 0; c < nc; ++c) {
        if (t->cell_bound_enc[c] < 0) continue;
        Data cd{1, c};
        const Grid& g = m.grid_of(cd);
        int nv = g.nv;
        double* fp = m.df(cd);
        double* vf = m.vsflux.data() + m.foff[c];
        double* w = m.w + (size_t)c * NW;
        double* pp = m.prim + (size_t)c * NW;
        double* wf = m.wflux.data() + (size_t)c * NW;
        const double* ds = t->cell_ds + (size_t)c * D;
        double area = ds[0];
        for (int d = 1; d < D; ++d) area *= ds[d];
        double prim_c[5], prim_n[5], wn[5], q[3];
        if (m.prm.marching == KG_MARCH_CAIDVM) {
            for (int e = 0; e < NW; ++e) w[e] += wf[e] * dt / area;
            get_prim(m, w, prim_c);
            double s = dt / area;
            for (size_t a = 0; a < (size_t)nv * NDF; ++a) fp[a] += s * vf[a];
            calc_w0(m, g, fp, wn);
            get_prim(m, wn, prim_n);
            double tau = get_tau(m, prim_c);
            double Fc[2], Fn[2];
            for (int i = 0; i < nv; ++i) {
                maxwell(m, g, i, prim_c, Fc);
                maxwell(m, g, i, prim_n, Fn);
                for (int k = 0; k < NDF; ++k) Model::F(fp, nv, i, k) += Fc[k] - Fn[k];
            }
            heat_flux(m, g, fp, prim_c, q);
            for (int e = 0; e < D; ++e) m.qf[(size_t)c * D + e] = q[e];
            double r1 = tau / (tau + dt), r2 = dt / (tau + dt);
            double Sp[2];
            for (int i = 0; i < nv; ++i) {
                maxwell(m, g, i, prim_c, Fc);
                shakhov(m, g, i, Fc, prim_c, q, Sp);
                for (int k = 0; k < NDF; ++k) {
                    double gplus = Fc[k] + Sp[k];
                    double v = Model::F(fp, nv, i, k) * r1;
                    Model::F(fp, nv, i, k) = v + r2 * gplus;
                }
            }
        } else if (m.prm.marching == KG_MARCH_CIP) {
            // w update, the positivity-preserving wall flux of a donor, convection, q of the
            // convected f, I-projection of f onto w, relaxation
            for (int e = 0; e < NW; ++e) w[e] += wf[e] * dt / area;
            if (t->cell_bound_enc[c] != 0) positivity_ib(m, c, area);
            get_prim(m, w, prim_c);
            double s = dt / area;
            for (size_t a = 0; a < (size_t)nv * NDF; ++a) fp[a] += s * vf[a];
            heat_flux(m, g, fp, prim_c, q);
            for (int e = 0; e < D; ++e) m.qf[(size_t)c * D + e] = q[e];
            double lam[5];
            conserved_iprojection(D, NDF, g.mid, g.weight, nv, fp, w, lam);
            double tau = get_tau(m, prim_c);
            double r1 = tau / (tau + dt), r2 = dt / (tau + dt);
            double Fc[2], Sp[2];
            for (int i = 0; i < nv; ++i) {
                maxwell(m, g, i, prim_c, Fc);
                shakhov(m, g, i, Fc, prim_c, q, Sp);
                for (int k = 0; k < NDF; ++k) {
                    double v = Model::F(fp, nv, i, k) * r1;
                    Model::F(fp, nv, i, k) = v + r2 * (Fc[k] + Sp[k]);
                }
            }
        } else {
            if (m.prm.flux == KG_FLUX_DVM) {
                calc_w0(m, g, fp, w);
            } else {
                for (int e = 0; e < NW; ++e) w[e] += wf[e] * dt / area;
            }
            get_prim(m, w, prim_c);
            double tau = get_tau(m, prim_c);
            heat_flux(m, g, fp, prim_c, q);
            for (int e = 0; e < D; ++e) m.qf[(size_t)c * D + e] = q[e];
            double s = dt / area, r1 = tau / (tau + dt), r2 = dt / (tau + dt);
            double Fc[2], Sp[2];
            for (int i = 0; i < nv; ++i) {
                maxwell(m, g, i, prim_c, Fc);
                shakhov(m, g, i, Fc, prim_c, q, Sp);
                for (int k = 0; k < NDF; ++k) {
                    double gplus = Fc[k] + Sp[k];
                    double fk = Model::F(fp, nv, i, k);
                    Model::F(fp, nv, i, k) = (fk + s * Model::F(vf, nv, i, k)) * r1 + r2 * gplus;
                }
            }
        }
        if (check) {
            for (int e = 0; e < NW; ++e) {
                double dlt = prim_c[e] - pp[e];
                res[(size_t)c * NW + e] = dlt * dlt;
                avg[(size_t)c * NW + e] = std::fabs(prim_c[e]);
            }
        }
        for (int e = 0; e < NW; ++e) pp[e] = prim_c[e];
        for (int e = 0; e < NW; ++e) wf[e] = 0.0;
        std::fill(vf, vf + (size_t)nv * NDF, 0.0);
    }
    if (check) {
        for (int e = 0; e < NW; ++e) { sum_res[e] = 0; sum_avg[e] = 0; }
        for (int c = 0; c < nc; ++c)
            for (int e = 0; e < NW; ++e) { sum_res[e] += res[(size_t)c * NW + e]; sum_avg[e] += avg[(size_t)c * NW + e]; }
    }
}

int setup(Model& m, const kg_params* prm, const kg_topology* t) {
    if (!prm || !t) { g_err = "null argument"; return KG_ERR_ARG; }
    m.prm = *prm;
    m.t = t;
    m.dim = t->dim;
    m.ndf = t->ndf;
    if (m.dim != prm->dim || m.ndf != prm->ndf) { g_err = "params/topology dim mismatch"; return KG_ERR_ARG; }
    m.grids.resize(t->n_grids);
    for (int g = 0; g < t->n_grids; ++g) {
        Grid& G = m.grids[g];
        G.off = t->grid_off[g];
        G.nv = (int)(t->grid_off[g + 1] - t->grid_off[g]);
        G.level = t->vs_level + G.off;
        G.weight = t->vs_weight + G.off;
        G.mid = t->vs_midpoint + G.off * m.dim;
    }
    int nc = t->n_cells;
    m.foff.resize(nc + 1);
    m.soff.resize(nc + 1);
    m.foff[0] = 0; m.soff[0] = 0;
    for (int c = 0; c < nc; ++c) {
        int nv = m.grids[t->cell_grid[c]].nv;
        m.foff[c + 1] = m.foff[c] + (int64_t)nv * m.ndf;
        m.soff[c + 1] = m.soff[c] + (int64_t)nv * m.ndf * m.dim;
    }
    m.wfoff.resize(t->n_walls + 1);
    m.wsoff.resize(t->n_walls + 1);
    m.wfoff[0] = 0; m.wsoff[0] = 0;
    for (int w = 0; w < t->n_walls; ++w) {
        int nv = m.grids[t->cell_grid[t->wall_donor[w]]].nv;
        m.wfoff[w + 1] = m.wfoff[w] + (int64_t)nv * m.ndf;
        m.wsoff[w + 1] = m.wsoff[w] + (int64_t)nv * m.ndf * m.dim;
    }
    m.vsflux.assign(m.foff[nc], 0.0);
    m.wflux.assign((size_t)nc * m.nw(), 0.0);
    return KG_OK;
}

}  // namespace

extern "C" {

// Size of the f array (doubles) and of the sdf array for a topology.
int kgo_sizes(const kg_topology* t, int64_t* nf, int64_t* nsdf, int64_t* nwall_f, int64_t* nwall_sdf) {
    int64_t a = 0, b = 0, c = 0, d = 0;
    for (int i = 0; i < t->n_cells; ++i) {
        int64_t nv = t->grid_off[t->cell_grid[i] + 1] - t->grid_off[t->cell_grid[i]];
        a += nv * t->ndf;
        b += nv * t->ndf * t->dim;
    }
    for (int w = 0; w < t->n_walls; ++w) {
        int g = t->cell_grid[t->wall_donor[w]];
        int64_t nv = t->grid_off[g + 1] - t->grid_off[g];
        c += nv * t->ndf;
        d += nv * t->ndf * t->dim;
    }
    *nf = a; *nsdf = b; *nwall_f = c; *nwall_sdf = d;
    return 0;
}

// Advance nsteps steps.  All state arrays are in/out.  wall_f / wall_sdf carry the
// SolidNeighbor distribution and boundary slope between steps (the reference keeps
// them in SolidNeighbor.vs_data); initialise wall_f with the donor's f and wall_sdf
// with zeros, as initialize_solid_neighbor! does (Immersed_boundary.jl:290-298).
int kgo_run(const kg_params* prm, const kg_topology* t, double dt, int64_t step0, int32_t nsteps,
            double* f, double* sdf, double* w, double* prim, double* qf, double* wall_f, double* wall_sdf,
            double* sum_res, double* sum_avg, int32_t* checked, int32_t nthreads) {
    Model m;
    int rc = setup(m, prm, t);
    if (rc) return rc;
    m.f = f; m.sdf = sdf; m.w = w; m.prim = prim; m.qf = qf; m.dt = dt;
    m.nthreads = nthreads < 1 ? 1 : nthreads;
    m.wall_f.assign(wall_f, wall_f + m.wfoff[t->n_walls]);
    m.wall_sdf.assign(wall_sdf, wall_sdf + m.wsoff[t->n_walls]);
    *checked = 0;
    try {
        for (int s = 0; s < nsteps; ++s) {
            int64_t step = step0 + s;
            slope(m);
            flux(m);
            double r[5], a[5];
            iterate(m, step, r, a);
            if (step % prm->st_check_interval == 0) {
                *checked = 1;
                for (int e = 0; e < m.nw(); ++e) { sum_res[e] = r[e]; sum_avg[e] = a[e]; }
            }
        }
    } catch (...) {
        return KG_ERR_TOPOLOGY;
    }
    std::copy(m.wall_f.begin(), m.wall_f.end(), wall_f);
    std::copy(m.wall_sdf.begin(), m.wall_sdf.end(), wall_sdf);
    return KG_OK;
}

// slope! alone (Flux/Slope.jl:1047-1070) on the state as it stands: the pass that
// ps_adaptive_mesh_refinement! (Physical_space/AMR.jl:1108-1116) runs before the criterion.
// sdf is overwritten; wall_f (the SolidNeighbor distributions) is read only.
int kgo_slope(const kg_params* prm, const kg_topology* t, const double* f, double* sdf, const double* wall_f,
              int32_t nthreads) {
    Model m;
    int rc = setup(m, prm, t);
    if (rc) return rc;
    m.f = const_cast<double*>(f); m.sdf = sdf;
    m.nthreads = nthreads < 1 ? 1 : nthreads;
    m.wall_f.assign(wall_f, wall_f + m.wfoff[t->n_walls]);
    m.wall_sdf.assign(m.wsoff[t->n_walls], 0.0);
    try {
        slope(m);
    } catch (...) {
        return KG_ERR_TOPOLOGY;
    }
    return KG_OK;
}

// save_result (IO/Output.jl:198-255) on the state as it stands: update_slope! and
// update_solid_cell! change the state (slopes, solid cells' df, w, prim), then per
// SolidNeighbor save_boundary_result! (Boundary/Immersed_boundary.jl:12-61) rebuilds the wall
// distribution at the aux point -- its wall-direction slope is written through the ssdf view,
// its df is a local -- and reports prim, qf (calc_w0, get_prim, calc_qf) and the pressure
// tensor (pressure_2D / pressure_3D, lib/KitCore/2D.jl:31-37, 3D.jl:37-46).
// rows: per wall record prim (dim+2), qf (dim), p (dim (dim+1) / 2).
int kgo_solution(const kg_params* prm, const kg_topology* t, double* f, double* sdf, double* w, double* prim,
                 double* wall_f, double* wall_sdf, double* rows, int32_t nthreads) {
    Model m;
    int rc = setup(m, prm, t);
    if (rc) return rc;
    m.f = f; m.sdf = sdf; m.w = w; m.prim = prim;
    std::vector<double> qdummy((size_t)std::max(1, t->n_cells * t->dim), 0.0);
    m.qf = qdummy.data();
    m.nthreads = nthreads < 1 ? 1 : nthreads;
    m.wall_f.assign(wall_f, wall_f + m.wfoff[t->n_walls]);
    m.wall_sdf.assign(wall_sdf, wall_sdf + m.wsoff[t->n_walls]);
    try {
        slope(m);
        update_solid_cells(m);
        const std::vector<double> kept = m.wall_f;
        update_walls(m);
        const int D = m.dim, NDF = m.ndf, NP = D * (D + 1) / 2, WR = 2 * D + 2 + NP;
        for (int wi = 0; wi < t->n_walls; ++wi) {
            Data cd{1, t->wall_donor[wi]}, wd{2, wi};
            const Grid& g = m.grid_of(cd);
            const double* df = m.df(wd);
            double wv[5], pv[5], q[3];
            calc_w0(m, g, df, wv);
            get_prim(m, wv, pv);
            heat_flux(m, g, df, pv, q);
            double* o = rows + (size_t)wi * WR;
            for (int e = 0; e < D + 2; ++e) o[e] = pv[e];
            for (int d = 0; d < D; ++d) o[D + 2 + d] = q[d];
            int e = 2 * D + 2;
            for (int a = 0; a < D; ++a)
                for (int b = a; b < D; ++b) {
                    double sum = 0.0;
                    for (int i = 0; i < g.nv; ++i) sum += g.u(i, a) * g.u(i, b) * df[i] * g.weight[i];
                    o[e++] = sum;
                }
            (void)NDF;
        }
        m.wall_f = kept;
    } catch (...) {
        return KG_ERR_TOPOLOGY;
    }
    std::copy(m.wall_f.begin(), m.wall_f.end(), wall_f);
    std::copy(m.wall_sdf.begin(), m.wall_sdf.end(), wall_sdf);
    return KG_OK;
}

// ---- physical-space adaptation: the state moves of ps_replace! (Physical_space/AMR.jl:633-703)
// vs_merge! (AMR.jl:343-366): the level merge walk adding the cells of grid n onto grid p --
// one-to-one on equal levels, finer cells over 2^(dim*Δl), a coarser cell into each cell it
// covers.  cols: the columns of the nv x cols block (ndf for df, ndf*dim for sdf).
static void vs_merge(int D, double* dst, const Grid& gp, const double* src, const Grid& gn, int cols) {
    int j = 0;
    double flag = 0.0;
    for (int i = 0; i < gp.nv; ++i) {
        const int li = gp.level[i];
        if (li == gn.level[j]) {
            for (int q = 0; q < cols; ++q) dst[(size_t)q * gp.nv + i] += src[(size_t)q * gn.nv + j];
            j += 1;
        } else if (li < gn.level[j]) {
            while (flag != 1.0) {
                const double div = std::ldexp(1.0, D * (gn.level[j] - li));
                for (int q = 0; q < cols; ++q) dst[(size_t)q * gp.nv + i] += src[(size_t)q * gn.nv + j] / div;
                flag += 1.0 / div;
                j += 1;
            }
            flag = 0.0;
        } else {
            for (int q = 0; q < cols; ++q) dst[(size_t)q * gp.nv + i] += src[(size_t)q * gn.nv + j];
            flag += 1.0 / std::ldexp(1.0, D * (li - gn.level[j]));
            if (flag == 1.0) { j += 1; flag = 0.0; }
        }
    }
}

// refine_grid_stream! / coarsen_grid_stream! (Velocity_space/Rebuild.jl:44-163), the df part:
// the new grid gn walked against the source grid go -- a velocity cell on both copied, the
// children of a refined cell each given its df, and 2^dim coarsened siblings merged as
// (Σ df) / 2^dim.  (A cover of mixed levels, which the streams never produce, is weighted by
// volume.)
static void vs_rebuild_df(int D, double* dst, const Grid& gn, const double* src, const Grid& go, int ndf) {
    int i = 0;
    for (int j = 0; j < gn.nv;) {
        const int ln = gn.level[j], lo = go.level[i];
        if (ln == lo) {
            for (int k = 0; k < ndf; ++k) dst[(size_t)k * gn.nv + j] = src[(size_t)k * go.nv + i];
            ++i; ++j;
        } else if (ln > lo) {
            double filled = 0.0;
            while (filled < 1.0) {
                for (int k = 0; k < ndf; ++k) dst[(size_t)k * gn.nv + j] = src[(size_t)k * go.nv + i];
                filled += 1.0 / std::ldexp(1.0, D * (gn.level[j] - lo));
                ++j;
            }
            ++i;
        } else {
            int i1 = i;
            bool same = true;
            double filled = 0.0;
            while (filled < 1.0) {
                same = same && go.level[i1] == ln + 1;
                filled += 1.0 / std::ldexp(1.0, D * (go.level[i1] - ln));
                ++i1;
            }
            for (int k = 0; k < ndf; ++k) {
                double s = 0.0;
                for (int q = i; q < i1; ++q)
                    s += same ? src[(size_t)k * go.nv + q] : src[(size_t)k * go.nv + q] / std::ldexp(1.0, D * (go.level[q] - ln));
                dst[(size_t)k * gn.nv + j] = same ? s / (1 << D) : s;
            }
            i = i1; ++j;
        }
    }
}

// The adapted mesh's state from the previous one, per new cell as src[c] says (see
// kg_adapt_src): KEEP copies; REFINE is ps_replace!(::Val{1}) applied depth times (ps_copy,
// ds halved, df += min(|df/(ds.|sdf| + EPS)|, 1) * (sdf . (ds/2 .* RMT[i])) with the parent's
// sdf, then calc_w0 and get_prim); COARSEN is ps_merge + vs_merge! of df and sdf over the
// children and the division by 2^dim.  qf of a replaced cell is zero (PsData's default).
// The *_old arrays are the previous state with the slopes of its current f (slope! runs
// before the replacements).
int kgo_adapt(const kg_params* prm, const kg_topology* told, const kg_topology* tnew, const kg_adapt_src* src,
              const double* f_old, const double* sdf_old, const double* w_old, const double* prim_old,
              const double* qf_old, double* f_new, double* sdf_new, double* w_new, double* prim_new, double* qf_new) {
    Model mo, mn;
    int rc = setup(mo, prm, told);
    if (rc) return rc;
    if ((rc = setup(mn, prm, tnew))) return rc;
    const int D = mn.dim, NDF = mn.ndf, NW = D + 2, nch = 1 << D;
    for (int c = 0; c < tnew->n_cells; ++c) {
        const kg_adapt_src& a = src[c];
        const Grid& g = mn.grids[tnew->cell_grid[c]];
        double* fn = f_new + mn.foff[c];
        double* sn = sdf_new + mn.soff[c];
        const size_t nf = (size_t)g.nv * NDF, ns = nf * D;
        if (a.kind == KG_ADAPT_KEEP) {
            const int o = a.src[0];
            std::copy(f_old + mo.foff[o], f_old + mo.foff[o] + nf, fn);
            std::copy(sdf_old + mo.soff[o], sdf_old + mo.soff[o] + ns, sn);
            for (int e = 0; e < NW; ++e) { w_new[(size_t)c * NW + e] = w_old[(size_t)o * NW + e]; prim_new[(size_t)c * NW + e] = prim_old[(size_t)o * NW + e]; }
            for (int d = 0; d < D; ++d) qf_new[(size_t)c * D + d] = qf_old[(size_t)o * D + d];
        } else if (a.kind == KG_ADAPT_REFINE) {
            const int o = a.src[0];
            std::copy(f_old + mo.foff[o], f_old + mo.foff[o] + nf, fn);
            std::copy(sdf_old + mo.soff[o], sdf_old + mo.soff[o] + ns, sn);
            double ds[3];
            for (int d = 0; d < D; ++d) ds[d] = told->cell_ds[(size_t)o * D + d];
            for (int l = 0; l < a.depth; ++l) {
                for (int d = 0; d < D; ++d) ds[d] *= 0.5;
                double off[3];
                for (int d = 0; d < D; ++d) off[d] = 0.5 * ds[d] * (((a.path[l] >> d) & 1) ? 1.0 : -1.0);
                for (int k = 0; k < NDF; ++k)
                    for (int j = 0; j < g.nv; ++j) {
                        double den = 0.0, dot = 0.0;
                        for (int d = 0; d < D; ++d) {
                            den += ds[d] * std::fabs(Model::S(sn, g.nv, NDF, j, k, d));
                            dot += Model::S(sn, g.nv, NDF, j, k, d) * off[d];
                        }
                        double& x = Model::F(fn, g.nv, j, k);
                        x += std::min(std::fabs(x / (den + EPS_REF)), 1.0) * dot;
                    }
            }
            calc_w0(mn, g, fn, w_new + (size_t)c * NW);
            get_prim(mn, w_new + (size_t)c * NW, prim_new + (size_t)c * NW);
            for (int d = 0; d < D; ++d) qf_new[(size_t)c * D + d] = 0.0;
        } else if (a.kind == KG_ADAPT_COARSEN) {
            double wsum[5];
            for (int e = 0; e < NW; ++e) {
                double s = w_old[(size_t)a.src[0] * NW + e];
                for (int q = 1; q < nch; ++q) s += w_old[(size_t)a.src[q] * NW + e];
                wsum[e] = s / nch;
                w_new[(size_t)c * NW + e] = wsum[e];
            }
            get_prim(mn, wsum, prim_new + (size_t)c * NW);
            std::fill(fn, fn + nf, 0.0);
            std::fill(sn, sn + ns, 0.0);
            for (int q = 0; q < nch; ++q) {
                const int o = a.src[q];
                const Grid& go = mo.grids[told->cell_grid[o]];
                vs_merge(D, sn, g, sdf_old + mo.soff[o], go, NDF * D);
                vs_merge(D, fn, g, f_old + mo.foff[o], go, NDF);
            }
            for (size_t e = 0; e < nf; ++e) fn[e] /= nch;
            for (size_t e = 0; e < ns; ++e) sn[e] /= nch;
            for (int d = 0; d < D; ++d) qf_new[(size_t)c * D + d] = 0.0;
        } else if (a.kind == KG_ADAPT_VS) {
            const int o = a.src[0];
            const Grid& go = mo.grids[told->cell_grid[o]];
            vs_rebuild_df(D, fn, g, f_old + mo.foff[o], go, NDF);
            std::fill(sn, sn + ns, 0.0);
            for (int e = 0; e < NW; ++e) { w_new[(size_t)c * NW + e] = w_old[(size_t)o * NW + e]; prim_new[(size_t)c * NW + e] = prim_old[(size_t)o * NW + e]; }
            for (int d = 0; d < D; ++d) qf_new[(size_t)c * D + d] = qf_old[(size_t)o * D + d];
        } else {
            g_err = "unknown adapt kind";
            return KG_ERR_ARG;
        }
    }
    return KG_OK;
}

// Moments (ρ, ρU, ρE) and heat flux of every cell's f relative to its prim
// (micro_to_macro / calc_qf), for the known-answer tests.
int kgo_moments(const kg_params* prm, const kg_topology* t, const double* f, const double* prim, double* w_out, double* q_out) {
    Model m;
    int rc = setup(m, prm, t);
    if (rc) return rc;
    for (int c = 0; c < t->n_cells; ++c) {
        const Grid& g = m.grids[t->cell_grid[c]];
        calc_w0(m, g, f + m.foff[c], w_out + (size_t)c * m.nw());
        heat_flux(m, g, f + m.foff[c], prim + (size_t)c * m.nw(), q_out + (size_t)c * m.dim);
    }
    return KG_OK;
}

// ---- physical-space criterion: update_criterion! (Physical_space/AMR.jl:1-284), the
// Löhner sensor of update_Lohner_inner_ps! (Physical_space/Criteria.jl:24-158) and the
// buffer layer of apply_amr_buffer! (AMR.jl:286-330), restated from the topology arrays.
static double jl_max(double a, double b) { return (std::isnan(a) || std::isnan(b)) ? NAN : (a > b ? a : b); }
static double o_lohner_value(double l, double c, double r, double dsL, double dsR, double eps) {
    const double scale = dsR * std::fabs(l) + (dsL + dsR) * std::fabs(c) + dsL * std::fabs(r);
    if (scale < 1e-4 * std::min(dsL, dsR)) return 0.0;
    const double denom = dsR * std::fabs(l - c) + dsL * std::fabs(r - c) + eps * scale;
    if (denom <= 0.0) return 0.0;
    return std::fabs(dsR * l - (dsL + dsR) * c + dsL * r) / denom;
}
static bool o_primitive_ok(double l, double c, double r) {
    const double jump = jl_max(std::fabs(l - c), std::fabs(r - c));
    return jump >= 1e-3 * jl_max(std::fabs(c), 1e-4);
}
// sw: (dim+2) x dim column-major; comp and dir 1-based as in the reference
static double o_velocity_slope(const double* sw, const double* prim, int nw, int comp, int dir) {
    const double* col = sw + (size_t)nw * (dir - 1);
    return (col[comp] - prim[comp] * col[0]) / prim[0];
}
static double o_vorticity(const double* sw, const double* prim, int D) {
    const int nw = D + 2;
    if (D == 2) return o_velocity_slope(sw, prim, nw, 1, 2) - o_velocity_slope(sw, prim, nw, 2, 1);
    const double c1 = o_velocity_slope(sw, prim, nw, 2, 3) - o_velocity_slope(sw, prim, nw, 3, 2);
    const double c2 = o_velocity_slope(sw, prim, nw, 3, 1) - o_velocity_slope(sw, prim, nw, 1, 3);
    const double c3 = o_velocity_slope(sw, prim, nw, 1, 2) - o_velocity_slope(sw, prim, nw, 2, 1);
    return std::sqrt(c1 * c1 + c2 * c2 + c3 * c3);
}
static bool o_vorticity_ok(double l, double c, double r, const double* prim, int D, double h) {
    double speed2 = 0.0;
    for (int i = 1; i <= D; ++i) speed2 += prim[i] * prim[i];
    const double lambda = jl_max(std::fabs(prim[D + 1]), 2.220446049250313e-16);
    const double vscale = jl_max(std::sqrt(speed2), 1.0 / std::sqrt(lambda));
    const double omega = jl_max(std::fabs(l), jl_max(std::fabs(c), std::fabs(r)));
    return omega * h >= 2e-2 * vscale;
}
static double o_sensor(const double* lo, int D) {
    double v = 0.0;
    for (int dir = 0; dir < D; ++dir) v = jl_max(v, jl_max(lo[(size_t)dir * (D + 2)], lo[(size_t)dir * (D + 2) + D + 1]));
    return v;
}

extern "C" int kgo_criterion(const kg_params* prm, const kg_topology* t, const double* w, const double* prim,
                             const double* sw, double thr, double* loh_out) {
    Model m;
    int rc = setup(m, prm, t);
    if (rc) return rc;
    const int D = t->dim, NW = D + 2, NF = 2 * D, N = NW * D;
    const int NC = t->n_cells;
    std::vector<double> lo((size_t)NC * N, 0.0);
    for (int c = 0; c < NC; ++c) {
        if (t->cell_bound_enc[c] < 0) continue;
        const double* pc = prim + (size_t)c * NW;
        const double* swc = sw + (size_t)c * N;
        const double omega_c = o_vorticity(swc, pc, D);
        for (int dir = 0; dir < D; ++dir) {
            double* row = lo.data() + (size_t)c * N + (size_t)dir * NW;
            const int s[2] = {t->nbr_state[c * NF + 2 * dir], t->nbr_state[c * NF + 2 * dir + 1]};
            if (s[0] == 0 || s[1] == 0) continue;                 // the Val{0} methods: zero row
            const double ds = t->cell_ds[(size_t)c * D + dir];
            double dss[2], pside[2][5], om[2];
            for (int side = 0; side < 2; ++side) {
                dss[side] = (s[side] == 1 ? 1.0 : (s[side] == -1 ? 1.5 : 0.75)) * ds;
                const int k = 2 * dir + side;
                const int32_t* lst = t->nbr_ref + t->nbr_off[c * NF + k];
                const int n = t->nbr_off[c * NF + k + 1] - t->nbr_off[c * NF + k];
                double ws[5] = {0, 0, 0, 0, 0};
                std::vector<double> sws(N, 0.0);
                // a SolidNeighbor's w and sw stay zero (Immersed_boundary.jl:300-302, 481-482)
                for (int j = 0; j < n; ++j) {
                    if (lst[j] < 0) continue;
                    for (int q = 0; q < NW; ++q) ws[q] += w[(size_t)lst[j] * NW + q];
                    for (int e = 0; e < N; ++e) sws[e] += sw[(size_t)lst[j] * N + e];
                }
                if (dss[side] > ds && lst[0] >= 0) {                // a coarser side
                    const int nb = lst[0];
                    for (int tr = 0; tr < D; ++tr) {
                        if (tr == dir) continue;
                        const double dx = t->cell_midpoint[(size_t)c * D + tr] - t->cell_midpoint[(size_t)nb * D + tr];
                        for (int q = 0; q < NW; ++q) ws[q] += dx * sw[(size_t)nb * N + (size_t)tr * NW + q];
                    }
                }
                for (int q = 0; q < NW; ++q) ws[q] /= n;
                for (int e = 0; e < N; ++e) sws[e] /= n;
                get_prim(m, ws, pside[side]);
                om[side] = o_vorticity(sws.data(), pside[side], D);
            }
            const bool use_vort = o_vorticity_ok(om[0], omega_c, om[1], pc, D, std::max(dss[0], dss[1]));
            const double eps_l = 0.2 * ds;
            for (int q = 0; q < NW; ++q) {
                if (q == 1) row[q] = use_vort ? o_lohner_value(om[0], omega_c, om[1], dss[0], dss[1], eps_l) : 0.0;
                else row[q] = o_primitive_ok(pside[0][q], pc[q], pside[1][q])
                                  ? o_lohner_value(pside[0][q], pc[q], pside[1][q], dss[0], dss[1], eps_l) : 0.0;
            }
        }
    }
    for (int c = 0; c < NC; ++c) {
        double* o = loh_out + (size_t)c * N;
        for (int e = 0; e < N; ++e) o[e] = lo[(size_t)c * N + e];
        if (t->cell_bound_enc[c] < 0 || o_sensor(lo.data() + (size_t)c * N, D) > thr) continue;
        bool flagged = false;
        for (int k = 0; k < NF && !flagged; ++k) {
            if (t->nbr_state[c * NF + k] == 0) continue;
            for (int j = t->nbr_off[c * NF + k]; j < t->nbr_off[c * NF + k + 1]; ++j) {
                const int32_t r = t->nbr_ref[j];
                if (r < 0 || t->cell_bound_enc[r] < 0) continue;
                if (o_sensor(lo.data() + (size_t)r * N, D) > thr) { flagged = true; break; }
            }
        }
        if (flagged) for (int e = 0; e < N; ++e) o[e] = 2.0 * thr;
    }
    return KG_OK;
}

// update_macro_slope! (Flux/Slope.jl:1022-1036): sw[:, dir] = calc_w0 of sdf[:, :, dir] for
// every cell with bound_enc >= 0; sw_out holds (dim+2) x dim doubles per cell (column-major,
// as PsData.sw); solid cells are left at zero.
int kgo_macro_slope(const kg_params* prm, const kg_topology* t, const double* sdf, double* sw_out) {
    Model m;
    int rc = setup(m, prm, t);
    if (rc) return rc;
    const int nw = m.nw(), D = m.dim;
    for (int c = 0; c < t->n_cells; ++c) {
        double* o = sw_out + (size_t)c * nw * D;
        for (int e = 0; e < nw * D; ++e) o[e] = 0.0;
        if (t->cell_bound_enc[c] < 0) continue;
        const Grid& g = m.grids[t->cell_grid[c]];
        for (int dir = 0; dir < D; ++dir)
            calc_w0(m, g, sdf + m.soff[c] + (size_t)g.nv * t->ndf * dir, o + (size_t)dir * nw);
    }
    return KG_OK;
}

int kgo_last_error(char* buf, size_t cap) {
    std::snprintf(buf, cap, "%s", g_err.c_str());
    return 0;
}

// conserved_I_porjection! of one velocity grid: df (column-major nv x ndf) in place, the
// multipliers λ (dim+2) out.  mid: column-major nv x dim midpoints, weight: nv.
int kgo_iprojection(int dim, int ndf, int nv, const double* mid, const double* weight, double* df, const double* w,
                    double* lam) {
    if ((dim != 2 || ndf != 2) && (dim != 3 || ndf != 1)) { g_err = "dim/ndf"; return KG_ERR_ARG; }
    if (nv <= 0 || !mid || !weight || !df || !w || !lam) { g_err = "null argument"; return KG_ERR_ARG; }
    conserved_iprojection(dim, ndf, mid, weight, nv, df, w, lam);
    return KG_OK;
}

}  // extern "C"

// ---- velocity-space adaptation flags: vs_refine! / vs_coarsen!'s per-velocity decisions
// (Velocity_space/AMR.jl:26-118, Criteria.jl:4-78,212-283, Neighbor.jl:74-204), restated on
// the topology arrays with the reference's own sorted-key index.
namespace {
constexpr int VS_INDEX_BITS = 24;
constexpr uint64_t VS_INDEX_MASK = (uint64_t(1) << VS_INDEX_BITS) - 1;
struct VsIndex {
    int D = 2, maxlevel = 0, mortonbits = 0;
    double vmin[3] = {0, 0, 0}, hf[3] = {0, 0, 0};
    long tn[3] = {1, 1, 1}, stride[3] = {1, 1, 1};
    std::vector<uint64_t> keys;
};
// build_vs_index! (Neighbor.jl:74-137)
void vs_build(VsIndex& ix, const Grid& g, int D, const double* vmin, const double* ds0, const int32_t* tn, int maxlevel) {
    ix.D = D; ix.maxlevel = maxlevel; ix.mortonbits = D * maxlevel;
    long s = 1;
    for (int d = 0; d < D; ++d) {
        ix.vmin[d] = vmin[d];
        ix.hf[d] = ds0[d] / std::ldexp(1.0, maxlevel);
        ix.tn[d] = tn[d];
        ix.stride[d] = s;
        s *= tn[d];
    }
    const long mask = (1L << maxlevel) - 1;
    ix.keys.resize(g.nv);
    for (int i = 0; i < g.nv; ++i) {
        const int L = g.level[i];
        long root_lin = 0;
        uint64_t morton = 0;
        for (int d = 0; d < D; ++d) {
            const double cell = ix.hf[d] * (double)(1L << (maxlevel - L));
            const long gi = (long)std::nearbyint((g.u(i, d) - 0.5 * cell - ix.vmin[d]) / ix.hf[d]);   // round, ties to even
            root_lin += (gi >> maxlevel) * ix.stride[d];
            const long q = gi & mask;
            for (int b = 0; b < maxlevel; ++b) morton |= (uint64_t)((q >> b) & 1) << (b * D + d);
        }
        const uint64_t cellkey = ((uint64_t)root_lin << ix.mortonbits) | morton;
        ix.keys[i] = (cellkey << VS_INDEX_BITS) | (uint64_t)(i + 1);
    }
    std::sort(ix.keys.begin(), ix.keys.end());
}
// _vs_locate_code (Neighbor.jl:139-151): 0-based leaf, or -1
int vs_locate_code(const VsIndex& ix, const Grid& g, uint64_t code) {
    const uint64_t packed = (code << VS_INDEX_BITS) | VS_INDEX_MASK;
    auto it = std::upper_bound(ix.keys.begin(), ix.keys.end(), packed);   // searchsortedlast
    if (it == ix.keys.begin()) return -1;
    --it;
    const uint64_t corner = *it >> VS_INDEX_BITS;
    const int leaf = (int)(*it & VS_INDEX_MASK) - 1;
    const uint64_t span = uint64_t(1) << (ix.D * (ix.maxlevel - g.level[leaf]));
    return (code >= corner && code < corner + span) ? leaf : -1;
}
// vs_face_neighbor (Neighbor.jl:181-204)
int vs_face_neighbor(const VsIndex& ix, const Grid& g, int i, int dim, int dir) {
    const long mask = (1L << ix.maxlevel) - 1;
    long root_lin = 0;
    uint64_t morton = 0;
    const int L = g.level[i];
    const double cell = ix.hf[dim] * (double)(1L << (ix.maxlevel - L));
    for (int d = 0; d < ix.D; ++d) {
        double coord = g.u(i, d);
        if (d == dim) coord += dir * (0.5 * cell + 0.5 * ix.hf[d]);
        const long gi = (long)std::floor((coord - ix.vmin[d]) / ix.hf[d]);
        if (gi < 0 || gi >= (ix.tn[d] << ix.maxlevel)) return -1;
        root_lin += (gi >> ix.maxlevel) * ix.stride[d];
        const long q = gi & mask;
        for (int b = 0; b < ix.maxlevel; ++b) morton |= (uint64_t)((q >> b) & 1) << (b * ix.D + d);
    }
    return vs_locate_code(ix, g, ((uint64_t)root_lin << ix.mortonbits) | morton);
}
double vs_cell_size(const VsIndex& ix, const Grid& g, int j, int d) { return ix.hf[d] * (double)(1L << (ix.maxlevel - g.level[j])); }
// _lohner_ratio (Criteria.jl:221-227)
double vs_lohner_ratio(double L, double C, double R, double dsL, double dsR, double eflt, double eabs, double scale) {
    const double num = std::fabs(dsR * L - (dsL + dsR) * C + dsL * R);
    const double den = dsR * std::fabs(L - C) + dsL * std::fabs(R - C) +
                       eflt * (dsR * std::fabs(L) + (dsL + dsR) * std::fabs(C) + dsL * std::fabs(R)) +
                       eabs * scale * (dsL + dsR);
    return den > 0 ? num / den : 0.0;
}
}  // namespace

extern "C" int kgo_vs_flags(const kg_params* prm, const kg_topology* t, const double* f, const double* sdf,
                            const double* w, const double* prim, const kg_vs_config* cfg, uint8_t* flags,
                            double* eta, double* vr_out) {
    Model m;
    int rc = setup(m, prm, t);
    if (rc) return rc;
    const int D = m.dim, NDF = m.ndf, NW = D + 2;
    double vmin[3] = {0, 0, 0}, ds0[3] = {0, 0, 0}, du[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) {
        vmin[d] = cfg->quadrature[2 * d];
        du[d] = cfg->quadrature[2 * d + 1] - cfg->quadrature[2 * d];
        ds0[d] = du[d] / cfg->vs_trees_num[d];
    }
    const int maxlevel = cfg->maxlevel;
    // vs_resolution (AMR.jl:139-166)
    double pdu = du[0], ptn = cfg->vs_trees_num[0];
    for (int d = 1; d < D; ++d) { pdu *= du[d]; ptn *= cfg->vs_trees_num[d]; }
    const double rweight = pdu / ptn / std::ldexp(1.0, D * maxlevel);
    double dens_res = 0.0, en_res = 0.0;
    for (int c = 0; c < t->n_cells; ++c) {
        if (t->cell_bound_enc[c] < 0) continue;
        const Grid& g = m.grids[t->cell_grid[c]];
        const double* fc = f + m.foff[c];
        const double* U = prim + (size_t)c * NW + 1;
        double dmax = -INFINITY, emax = -INFINITY;
        for (int k = 0; k < NDF; ++k)
            for (int i = 0; i < g.nv; ++i) dmax = std::max(dmax, fc[(size_t)k * g.nv + i]);
        for (int i = 0; i < g.nv; ++i) {
            double c2 = 0.0;
            for (int d = 0; d < D; ++d) { const double x = U[d] - g.u(i, d); c2 += x * x; }
            const double e = NDF == 1 ? fc[i] * c2 : fc[i] * c2 + fc[g.nv + i];
            emax = std::max(emax, e);
        }
        dens_res = std::max(dmax * rweight, dens_res);
        en_res = std::max(0.5 * emax * rweight, en_res);
    }
    if (vr_out) { vr_out[0] = dens_res; vr_out[1] = en_res; }
    const bool lohner = cfg->mode == KG_VS_LOHNER;
    const double tauL = cfg->coeffi_lohner, tauC = 0.3 * cfg->coeffi_lohner;
    const double cl = cfg->coeffi_local, cg = cfg->coeffi_global;
    const double nch = std::ldexp(1.0, D);
    VsIndex ix;
    int64_t row = 0;
    for (int c = 0; c < t->n_cells; ++c) {
        const Grid& g = m.grids[t->cell_grid[c]];
        const double* fc = f + m.foff[c];
        const double* sc = sdf + m.soff[c];
        const double* wc = w + (size_t)c * NW;
        const double* U = prim + (size_t)c * NW + 1;
        const double* ds = t->cell_ds + (size_t)c * D;
        double s1 = 0.0, s2 = 0.0;
        if (lohner) {
            vs_build(ix, g, D, vmin, ds0, cfg->vs_trees_num, maxlevel);
            for (int i = 0; i < g.nv; ++i) {
                const double a1 = std::fabs(fc[i]);
                if (a1 > s1) s1 = a1;
                if (NDF == 2) { const double a2 = std::fabs(fc[g.nv + i]); if (a2 > s2) s2 = a2; }
            }
        }
        double U2 = 0.0;
        for (int d = 0; d < D; ++d) U2 += U[d] * U[d];
        const double den = wc[NW - 1] - 0.5 * wc[0] * U2;
        for (int i = 0; i < g.nv; ++i) {
            // _criterion_cell! (AMR.jl:8-20)
            double cdf[2];
            for (int k = 0; k < NDF; ++k) {
                double mm = 0.0;
                for (int d = 0; d < D; ++d) {
                    const double a = std::fabs(Model::S(const_cast<double*>(sc), g.nv, NDF, i, k, d) * ds[d]);
                    if (a > mm) mm = a;
                }
                cdf[k] = fc[(size_t)k * g.nv + i] + mm;
            }
            double S = 0.0;
            for (int d = 0; d < D; ++d) { const double x = U[d] - g.u(i, d); S += x * x; }
            const double wt = g.weight[i];
            const double en = NDF == 2 ? 0.5 * (S * cdf[0] + cdf[1]) * wt : 0.5 * S * cdf[0] * wt;
            const double rho = cdf[0] * wt;
            const bool loc_ref = std::max(std::fabs(en) / den, rho / wc[0]) > cl;
            const bool loc_coa = std::max(en / den, rho / wc[0]) < cl / nch;
            const bool glo_ref = rho > cg * dens_res || en > en_res * cg;
            const bool glo_coa = rho < cg * dens_res / nch && en < en_res * cg / nch;
            double e = 0.0;
            if (lohner) {
                // vs_lohner_indicator (Criteria.jl:253-283)
                const double h0 = fc[i], b0 = NDF == 2 ? fc[g.nv + i] : 0.0;
                for (int d = 0; d < D; ++d) {
                    const double hi = vs_cell_size(ix, g, i, d);
                    const int Ln = vs_face_neighbor(ix, g, i, d, -1), Rn = vs_face_neighbor(ix, g, i, d, +1);
                    const double dsL = Ln < 0 ? hi : 0.5 * (hi + vs_cell_size(ix, g, Ln, d));
                    const double dsR = Rn < 0 ? hi : 0.5 * (hi + vs_cell_size(ix, g, Rn, d));
                    const double hL = Ln < 0 ? 0.0 : fc[Ln], hR = Rn < 0 ? 0.0 : fc[Rn];
                    e = std::max(e, vs_lohner_ratio(hL, h0, hR, dsL, dsR, 1e-2, 1e-3, s1));
                    if (NDF == 2) {
                        const double bL = Ln < 0 ? 0.0 : fc[g.nv + Ln], bR = Rn < 0 ? 0.0 : fc[g.nv + Rn];
                        e = std::max(e, vs_lohner_ratio(bL, b0, bR, dsL, dsR, 1e-2, 1e-3, s2));
                    }
                }
            }
            const bool refine = g.level[i] < maxlevel && (lohner ? (e > tauL || loc_ref) : (loc_ref || glo_ref));
            const bool coarsen = lohner ? (e < tauC && loc_coa) : (loc_coa && glo_coa);
            flags[row + i] = (uint8_t)((refine ? 1 : 0) | (coarsen ? 2 : 0));
            if (eta) eta[row + i] = e;
        }
        row += g.nv;
    }
    return KG_OK;
}
