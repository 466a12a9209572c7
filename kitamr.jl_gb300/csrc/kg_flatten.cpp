// kg_flatten.cpp -- host flattener: reference-shaped kg_topology -> gather form.
//
// The decisions the reference takes per cell and direction while it walks its
// objects (slope dispatch on neighbour states, transverse projection flags, the
// per-face upwind split, which side of a face is updated) depend only on topology,
// so they are taken here once per adaptation and handed to the kernels as tables.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <unordered_map>
#include <utility>
#include "kg_internal.h"

namespace kg {
namespace {

struct Ctx {
    const kg_topology* t;
    int D, NDF;
    Flat* F;
    PairIds* pid;
    std::string* err;
};

int grid_nv(const kg_topology& t, int g) { return (int)(t.grid_off[g + 1] - t.grid_off[g]); }

}  // namespace

// The reference's level merge walk (diff_vs!, Flux/Slope.jl:36-63; vs_merge!,
// Physical_space/AMR.jl:343-366) defines, for every velocity cell i of grid A, the run of
// grid-B cells that overlap it: one cell when B is as coarse or coarser there, the whole
// covering run when B is finer.  runs receives (j0, count) per cell of A.
bool level_runs(const int8_t* la, int na, const int8_t* lb, int nb, int D, std::vector<int32_t>& runs) {
    runs.clear();
    runs.reserve((size_t)2 * na);
    int j = 0;
    double flag = 0.0;
    for (int i = 0; i < na; ++i) {
        if (j >= nb) return false;
        const int li = la[i];
        if (li == lb[j]) {
            runs.push_back(j); runs.push_back(1);
            j += 1;
        } else if (li < lb[j]) {
            int j0 = j, cnt = 0;
            while (flag != 1.0) {
                if (j >= nb) return false;
                flag += 1.0 / std::ldexp(1.0, D * (lb[j] - li));
                j += 1; cnt += 1;
            }
            flag = 0.0;
            runs.push_back(j0); runs.push_back(cnt);
        } else {
            runs.push_back(j); runs.push_back(1);
            flag += 1.0 / std::ldexp(1.0, D * (li - lb[j]));
            if (flag == 1.0) { j += 1; flag = 0.0; }
        }
    }
    return j == nb;
}

namespace {

// data index of a neighbour reference (cells first, then walls); -1 for none/inside
int data_of(const Ctx& c, int32_t r) {
    if (r == KG_NBR_NONE || r == KG_NBR_INSIDE) return -1;
    if (r >= 0) return r;
    return c.t->n_cells + (-1 - r);
}

// the pairing id of (my grid ga <- its grid gb): -1 for the same grid (identity), -2 when the
// canonical table has no such pair (a reference the pair scan did not see: a malformed list)
int pairing(Ctx& c, int ga, int gb) {
    if (ga == gb) return -1;
    const int id = c.pid->find(ga, gb);
    if (id < 0) { *c.err = "velocity pairing missing for a referenced grid pair"; return -2; }
    return id;
}

const double* dmid(const Ctx& c, int d) { return &c.F->dmid[(size_t)d * MAXD]; }


// data index of a neighbour reference without a context
int data_ref(const kg_topology& t, int32_t r) {
    if (r == KG_NBR_NONE || r == KG_NBR_INSIDE) return -1;
    if (r >= 0) return r < t.n_cells ? r : -1;
    const int w = -1 - r;
    return w < t.n_walls ? t.n_cells + w : -1;
}

}  // namespace

int PairIds::find(int ga, int gb) const {
    if (!dense.empty()) return dense[(size_t)ga * G + gb];
    auto it = ids.find(std::make_pair(ga, gb));
    return it == ids.end() ? -1 : it->second;
}

// The velocity pairings of a topology in one canonical order: every (my grid, its grid) pair,
// in both directions, that a neighbour reference, an inner face or a wall record relates,
// numbered by ascending (my grid, its grid).  The host and the device builders of the gather
// form look pairings up here, so both give every reference the same id.
int build_pairs(const kg_topology& t, Flat& F, PairIds& pid, std::string& err) {
    const int G = t.n_grids, NC = t.n_cells, NF = 2 * t.dim;
    pid.G = G;
    std::vector<uint8_t> mark;
    std::set<std::pair<int, int>> sp;
    if (G <= 1024) mark.assign((size_t)G * G, 0);
    auto add = [&](int ga, int gb) {
        if (ga == gb) return;
        if (!mark.empty()) { mark[(size_t)ga * G + gb] = 1; mark[(size_t)gb * G + ga] = 1; }
        else { sp.insert(std::make_pair(ga, gb)); sp.insert(std::make_pair(gb, ga)); }
    };
    for (int i = 0; i < NC; ++i) {
        const int gi = t.cell_grid[i];
        for (int32_t r = t.nbr_off[i * NF]; r < t.nbr_off[(i + 1) * NF]; ++r) {
            const int dn = data_ref(t, t.nbr_ref[r]);
            if (dn >= 0) add(gi, F.dgrid[dn]);
        }
    }
    for (int fi = 0; fi < t.n_faces; ++fi) {
        if (t.face_kind[fi] == KG_FACE_DOMAIN) continue;
        const int here = t.face_here[fi], od = data_ref(t, t.face_there[fi]);
        if (here >= 0 && here < NC && od >= 0) add(t.cell_grid[here], F.dgrid[od]);
    }
    for (int w = 0; w < t.n_walls; ++w) add(t.cell_grid[t.wall_donor[w]], t.cell_grid[t.wall_solid[w]]);
    std::vector<std::pair<int, int>> order;
    if (!mark.empty()) {
        for (int a = 0; a < G; ++a)
            for (int b = 0; b < G; ++b)
                if (mark[(size_t)a * G + b]) order.push_back(std::make_pair(a, b));
        pid.dense.assign((size_t)G * G, -1);
    } else {
        order.assign(sp.begin(), sp.end());
    }
    F.p_off.assign(1, 0);
    std::vector<int32_t> runs;
    for (size_t q = 0; q < order.size(); ++q) {
        const int ga = order[q].first, gb = order[q].second;
        if (!level_runs(t.vs_level + t.grid_off[ga], grid_nv(t, ga), t.vs_level + t.grid_off[gb], grid_nv(t, gb), t.dim, runs)) {
            err = "velocity grids do not tile the same root lattice";
            return KG_ERR_TOPOLOGY;
        }
        for (size_t r = 0; r < runs.size(); r += 2) { F.p_j0.push_back(runs[r]); F.p_cnt.push_back(runs[r + 1]); }
        F.p_off.push_back((int64_t)F.p_j0.size());
        if (!pid.dense.empty()) pid.dense[(size_t)ga * G + gb] = (int32_t)q;
        else pid.ids[order[q]] = (int)q;
    }
    return KG_OK;
}

// Empties a gather form but keeps the capacity of its arrays: rebuilding one of a similar size
// (the next adaptation, the next merge) then touches no fresh pages, whose first-touch faults
// cost more than filling ~20 MB of records.
void reset(Flat& F) {
    static_assert(sizeof(Flat) == 51 * sizeof(std::vector<int32_t>) + 64, "a Flat member was added or removed: reset it here");
    F.devlay = false;
    F.dim = 2; F.ndf = 2; F.n_cells = 0; F.n_walls = 0; F.n_data = 0; F.n_fluid = 0; F.phase_cells = 0;
    F.max_nv = 0; F.max_axis = 0; F.max_inc = 0; F.max_bcm = 0;
    F.g_off.clear(); F.vlev.clear(); F.vw.clear(); F.vu.clear(); F.vuf.clear(); F.vwf.clear();
    F.ax_off.clear(); F.ax_val.clear(); F.ax_hi.clear(); F.ax_lo.clear(); F.vidx.clear();
    F.foff.clear(); F.dgrid.clear(); F.dbe.clear(); F.dinvv.clear(); F.dnv.clear(); F.dprob.clear();
    F.dmid.clear(); F.dds.clear();
    F.p_off.clear(); F.p_j0.clear(); F.p_cnt.clear();
    F.pass_off.clear(); F.slope_ops.clear(); F.pass_cells_off.clear(); F.pass_cells.clear();
    F.cell_slope_op.clear(); F.slope_nbr.clear(); F.slope_items.clear(); F.pass_items_off.clear();
    F.fluid_cells.clear(); F.fcrec.clear(); F.regrec.clear(); F.fluid_r2.clear(); F.r2rec.clear(); F.screc.clear(); F.crit_ops.clear(); F.crit_nbr.clear();
    F.fluid_reg.clear();
    F.inc_off.clear(); F.inc.clear(); F.bc_prim.clear(); F.bc_hl.clear();
    F.solid_ops.clear(); F.wall_ops.clear(); F.ib_nbr.clear(); F.ib_dx.clear(); F.cut_idx.clear();
    F.cut_gw.clear(); F.cut_sw.clear(); F.cvcw.clear();
}

int flatten_head(const kg_params& prm, const kg_topology& t, Flat& F, PairIds& pid, std::string& err) {
    reset(F);
    pid.clear();
    if (t.dim != 2 && t.dim != 3) { err = "dim must be 2 or 3"; return KG_ERR_ARG; }
    if (t.ndf != (t.dim == 2 ? 2 : 1)) { err = "ndf must be 2 in 2D and 1 in 3D"; return KG_ERR_ARG; }
    if (prm.dim != t.dim || prm.ndf != t.ndf) { err = "params and topology disagree on dim/ndf"; return KG_ERR_ARG; }
    if (prm.st_check_interval <= 0) { err = "st_check_interval must be positive"; return KG_ERR_ARG; }
    if (t.n_grids <= 0 || t.n_cells <= 0) { err = "empty topology"; return KG_ERR_TOPOLOGY; }
    if (!t.grid_off || !t.vs_level || !t.vs_weight || !t.vs_midpoint || !t.cell_bound_enc || !t.cell_level ||
        !t.cell_grid || !t.cell_midpoint || !t.cell_ds || !t.nbr_state || !t.nbr_off || !t.nbr_ref ||
        (t.n_faces > 0 && (!t.face_kind || !t.face_dir || !t.face_rot || !t.face_area || !t.face_midpoint ||
                           !t.face_here || !t.face_there || !t.face_there_midpoint || !t.face_bc_kind || !t.face_bc)) ||
        (t.n_walls > 0 && (!t.wall_donor || !t.wall_solid || !t.wall_faceid || !t.wall_aux_point ||
                           !t.wall_normal || !t.wall_bc || !t.wall_cut_off)))
        { err = "null topology array"; return KG_ERR_ARG; }
    const int D = t.dim, NDF = t.ndf, NC = t.n_cells, NWL = t.n_walls;
    F.dim = D; F.ndf = NDF; F.n_cells = NC; F.n_walls = NWL; F.n_data = NC + NWL;

    // ---- velocity grids ------------------------------------------------------
    int64_t PG = t.grid_off[t.n_grids];
    if (t.grid_off[0] != 0 || PG <= 0) { err = "grid_off must start at 0"; return KG_ERR_TOPOLOGY; }
    for (int g = 0; g < t.n_grids; ++g) {
        if (t.grid_off[g + 1] <= t.grid_off[g]) { err = "empty velocity grid"; return KG_ERR_TOPOLOGY; }
        F.max_nv = std::max(F.max_nv, grid_nv(t, g));
    }
    F.g_off.assign(t.grid_off, t.grid_off + t.n_grids + 1);
    F.vlev.assign(t.vs_level, t.vs_level + PG);
    F.vw.assign(t.vs_weight, t.vs_weight + PG);
    F.vu.assign((size_t)D * PG, 0.0);
    for (int g = 0; g < t.n_grids; ++g) {
        int nv = grid_nv(t, g);
        const double* m = t.vs_midpoint + t.grid_off[g] * D;
        for (int d = 0; d < D; ++d)
            for (int i = 0; i < nv; ++i) F.vu[(size_t)d * PG + t.grid_off[g] + i] = m[(size_t)d * nv + i];
        // v = 0 must lie on a root corner (check_vs_setting, Solver/Types.jl:335-353):
        // no midpoint may have a zero component, or the upwind split would be ambiguous
        for (int d = 0; d < D; ++d)
            for (int i = 0; i < nv; ++i)
                if (m[(size_t)d * nv + i] == 0.0) { err = "a velocity midpoint lies on u_d = 0 (v = 0 must be a root corner)"; return KG_ERR_TOPOLOGY; }
    }

    F.vuf.assign(F.vu.begin(), F.vu.end());
    F.vwf.assign(F.vw.begin(), F.vw.end());
    // axis tables: exp(-λ|u-U|²) = Π_d exp(-λ(u_d-U_d)²), so a Maxwellian on a grid needs the
    // 1D factors at the distinct coordinates only
    F.ax_off.assign((size_t)t.n_grids * MAXD + 1, 0);
    F.vidx.assign((size_t)D * PG, 0);
    for (int g = 0; g < t.n_grids; ++g) {
        int nv = grid_nv(t, g);
        for (int d = 0; d < MAXD; ++d) {
            size_t slot = (size_t)g * MAXD + d;
            F.ax_off[slot] = (int32_t)F.ax_val.size();
            if (d < D) {
                std::vector<double> vals(F.vu.begin() + (size_t)d * PG + t.grid_off[g],
                                         F.vu.begin() + (size_t)d * PG + t.grid_off[g] + nv);
                std::sort(vals.begin(), vals.end());
                vals.erase(std::unique(vals.begin(), vals.end()), vals.end());
                if (vals.size() > 65535) { err = "more than 65535 distinct velocity coordinates on an axis"; return KG_ERR_TOPOLOGY; }
                F.max_axis = std::max(F.max_axis, (int)vals.size());
                for (int i = 0; i < nv; ++i) {
                    double x = F.vu[(size_t)d * PG + t.grid_off[g] + i];
                    F.vidx[(size_t)d * PG + t.grid_off[g] + i] = (uint16_t)(std::lower_bound(vals.begin(), vals.end(), x) - vals.begin());
                }
                F.ax_val.insert(F.ax_val.end(), vals.begin(), vals.end());
                for (double x : vals) {
                    const float hi = (float)x;
                    F.ax_hi.push_back(hi);
                    F.ax_lo.push_back((float)(x - (double)hi));
                }
            }
            F.ax_off[slot + 1] = (int32_t)F.ax_val.size();
        }
    }

    // ---- data table: cells then walls -------------------------------------------
    F.foff.assign(F.n_data + 1, 0);
    F.dgrid.resize(F.n_data); F.dbe.resize(F.n_data);
    F.dmid.assign((size_t)F.n_data * MAXD, 0.0); F.dds.assign((size_t)F.n_data * MAXD, 0.0);
    for (int i = 0; i < NC; ++i) {
        int g = t.cell_grid[i];
        if (g < 0 || g >= t.n_grids) { err = "cell_grid out of range"; return KG_ERR_TOPOLOGY; }
        F.dgrid[i] = g; F.dbe[i] = t.cell_bound_enc[i];
        for (int d = 0; d < D; ++d) { F.dmid[(size_t)i * MAXD + d] = t.cell_midpoint[(size_t)i * D + d]; F.dds[(size_t)i * MAXD + d] = t.cell_ds[(size_t)i * D + d]; }
    }
    for (int w = 0; w < NWL; ++w) {
        int dn = t.wall_donor[w], sc = t.wall_solid[w];
        if (dn < 0 || dn >= NC || sc < 0 || sc >= NC) { err = "wall donor/solid out of range"; return KG_ERR_TOPOLOGY; }
        if (t.cell_bound_enc[dn] <= 0 || t.cell_bound_enc[sc] >= 0) { err = "wall donor must have bound_enc > 0 and solid bound_enc < 0"; return KG_ERR_TOPOLOGY; }
        int i = NC + w;
        F.dgrid[i] = t.cell_grid[dn];              // SolidNeighbor shares the donor's grid
        F.dbe[i] = t.cell_bound_enc[sc];           // and the solid cell's bound_enc, midpoint, ds
        for (int d = 0; d < D; ++d) { F.dmid[(size_t)i * MAXD + d] = t.cell_midpoint[(size_t)sc * D + d]; F.dds[(size_t)i * MAXD + d] = t.cell_ds[(size_t)sc * D + d]; }
    }
    for (int i = 0; i < F.n_data; ++i) F.foff[i + 1] = F.foff[i] + (int64_t)grid_nv(t, F.dgrid[i]) * NDF;
    F.dinvv.resize(F.n_data);
    for (int i = 0; i < F.n_data; ++i) {
        double v = F.dds[(size_t)i * MAXD];
        for (int d = 1; d < D; ++d) v *= F.dds[(size_t)i * MAXD + d];
        F.dinvv[i] = 1.0 / v;
    }
    F.dnv.resize(F.n_data);
    F.dprob.assign(F.n_data, 0);
    for (int i = 0; i < F.n_data; ++i) F.dnv[i] = grid_nv(t, F.dgrid[i]);

    // ---- neighbour access helpers ---------------------------------------------------
    const int NF = 2 * D;
    int64_t nref = t.nbr_off[NC * NF];
    for (int i = 0; i < NC * NF; ++i)
        if (t.nbr_off[i + 1] < t.nbr_off[i] || (t.nbr_off[i + 1] == t.nbr_off[i])) { err = "empty neighbour list (a boundary list holds one KG_NBR_NONE)"; return KG_ERR_TOPOLOGY; }
    for (int64_t r = 0; r < nref; ++r) {
        int32_t v = t.nbr_ref[r];
        if (v >= NC || (v < 0 && v != KG_NBR_NONE && v != KG_NBR_INSIDE && (-1 - v) >= NWL)) { err = "nbr_ref out of range"; return KG_ERR_TOPOLOGY; }
    }
    // fluid cells: count, phase cells, levels
    int Lmin = INT32_MAX, Lmax = 0;
    for (int i = 0; i < NC; ++i) {
        if (t.cell_bound_enc[i] < 0) continue;
        F.n_fluid++;
        F.phase_cells += grid_nv(t, t.cell_grid[i]);
        Lmin = std::min(Lmin, t.cell_level[i]);
        Lmax = std::max(Lmax, t.cell_level[i]);
    }
    if (F.n_fluid == 0) { err = "no fluid cells"; return KG_ERR_TOPOLOGY; }
    pid.lmin = Lmin;
    pid.lmax = Lmax;
    return build_pairs(t, F, pid, err);
}

// The checks of the face list that the host builder makes while it places the incidences, in
// its order and with its messages (the device builder runs them here first).
int flatten_checks(const kg_params& prm, const kg_topology& t, const Flat& F, std::string& err) {
    const int D = t.dim, NC = t.n_cells;
    for (int fi = 0; fi < t.n_faces; ++fi) {
        const int here = t.face_here[fi];
        if (here < 0 || here >= NC) { err = "face here side must be a fluid cell"; return KG_ERR_TOPOLOGY; }
    }
    for (int fi = 0; fi < t.n_faces; ++fi) {
        const int dir = t.face_dir[fi];
        if (dir < 0 || dir >= D) { err = "face_dir out of range"; return KG_ERR_TOPOLOGY; }
        const int here = t.face_here[fi];
        if (t.cell_bound_enc[here] < 0) { err = "face here side must be a fluid cell"; return KG_ERR_TOPOLOGY; }
        const double rot = t.face_rot[fi];
        if (rot != 1.0 && rot != -1.0) { err = "face_rot must be +1 or -1"; return KG_ERR_TOPOLOGY; }
        if (t.face_kind[fi] == KG_FACE_DOMAIN) {
            const int bk = t.face_bc_kind[fi];
            if (bk < KG_BC_MAXWELL || bk > KG_BC_INTERP) { err = "unknown domain boundary kind"; return KG_ERR_TOPOLOGY; }
            if (bk == KG_BC_MAXWELL && prm.flux == KG_FLUX_DVM) { err = "DVM Maxwellian domain flux is undefined in the reference (DVM.jl:3,12)"; return KG_ERR_TOPOLOGY; }
            if (bk == KG_BC_INTERP && D != 2) { err = "InterpolatedOutflow is 2D only in the reference"; return KG_ERR_TOPOLOGY; }
            continue;
        }
        const int od = data_ref(t, t.face_there[fi]);
        if (od < 0) { err = "inner face without a there side"; return KG_ERR_TOPOLOGY; }
        if (F.dbe[od] < 0 && od >= NC && F.dgrid[od] != t.cell_grid[here]) { err = "wall grid differs from donor grid"; return KG_ERR_TOPOLOGY; }
    }
    return KG_OK;
}

// The immersed-boundary records (update_solid_cell!, Boundary/Immersed_boundary.jl:122-146;
// update_solid_neighbor!, :367-500): the solid cells' extrapolation sources and the wall
// records' image sources, cut cells and weights.
int flatten_ib(const kg_topology& t, Flat& F, const PairIds& pid, std::string& err) {
    const int D = t.dim, NC = t.n_cells, NWL = t.n_walls, NF = 2 * D;
    Ctx c{&t, D, t.ndf, &F, const_cast<PairIds*>(&pid), &err};
    auto lst = [&](int cell, int k) { return t.nbr_ref + t.nbr_off[cell * NF + k]; };
    // ---- immersed boundary (Boundary/Immersed_boundary.jl:122-146,367-500) -----------------
    auto fluid_sources = [&](int cell, const double* target, std::vector<int>& srcs) {
        for (int k = 0; k < NF; ++k) {
            int32_t r = lst(cell, k)[0];
            if (r >= 0 && t.cell_bound_enc[r] >= 0) srcs.push_back(r);
        }
        (void)target;
    };
    auto push_sources = [&](int tgt_grid, const std::vector<int>& srcs, const double* target) -> int {
        for (int s : srcs) {
            int p = pairing(c, tgt_grid, t.cell_grid[s]);
            if (p == -2) return KG_ERR_TOPOLOGY;
            F.ib_nbr.push_back(NbrRef{s, p});
            for (int d = 0; d < MAXD; ++d) F.ib_dx.push_back(d < D ? target[d] - t.cell_midpoint[(size_t)s * D + d] : 0.0);
        }
        return KG_OK;
    };
    for (int i = 0; i < NC; ++i) {
        if (t.cell_bound_enc[i] >= 0) continue;
        std::vector<int> srcs;
        const double* tm = t.cell_midpoint + (size_t)i * D;
        fluid_sources(i, tm, srcs);
        SolidOp so{};
        so.cell = i; so.list = (int32_t)F.ib_nbr.size(); so.cnt = (int32_t)srcs.size();
        if (srcs.empty()) { err = "solid cell without fluid neighbours"; return KG_ERR_TOPOLOGY; }
        int rc = push_sources(t.cell_grid[i], srcs, tm);
        if (rc) return rc;
        F.solid_ops.push_back(so);
    }
    for (int w = 0; w < NWL; ++w) {
        WallOp wo{};
        int dn = t.wall_donor[w], sc = t.wall_solid[w];
        int k = t.wall_faceid[w];
        if (k < 0 || k >= NF) { err = "wall faceid out of range"; return KG_ERR_TOPOLOGY; }
        wo.donor = dn; wo.solid = sc; wo.data = NC + w; wo.dir = k / 2;
        for (int d = 0; d < D; ++d) {
            wo.aux[d] = t.wall_aux_point[(size_t)w * D + d];
            wo.normal[d] = t.wall_normal[(size_t)w * D + d];
            wo.ib_point[d] = wo.aux[d] + t.cell_midpoint[(size_t)dn * D + d] - t.cell_midpoint[(size_t)sc * D + d];
        }
        for (int e = 0; e < D + 2; ++e) wo.bc[e] = t.wall_bc[(size_t)w * (D + 2) + e];
        int dir = wo.dir;
        wo.dxf = wo.ib_point[dir] - t.cell_midpoint[(size_t)dn * D + dir];
        wo.dxs = t.cell_midpoint[(size_t)dn * D + dir] - t.cell_midpoint[(size_t)sc * D + dir];
        wo.dxL = wo.aux[dir] - wo.ib_point[dir];
        std::vector<int> srcs;
        fluid_sources(dn, wo.ib_point, srcs);
        srcs.push_back(dn);  // image_df appends the donor itself (Immersed_boundary.jl:373)
        wo.list = (int32_t)F.ib_nbr.size(); wo.cnt = (int32_t)srcs.size();
        int rc = push_sources(t.cell_grid[dn], srcs, wo.ib_point);
        if (rc) return rc;
        wo.spair = pairing(c, t.cell_grid[dn], t.cell_grid[sc]);
        if (wo.spair == -2) return KG_ERR_TOPOLOGY;
        int c0 = t.wall_cut_off[w], c1 = t.wall_cut_off[w + 1];
        if (c1 < c0) { err = "wall_cut_off must be non-decreasing"; return KG_ERR_TOPOLOGY; }
        wo.cut_off = (int32_t)F.cut_idx.size(); wo.cut_cnt = c1 - c0;
        int nv = grid_nv(t, t.cell_grid[dn]);
        wo.cvcw_off = (int64_t)F.cvcw.size();
        const double* wt = t.vs_weight + t.grid_off[t.cell_grid[dn]];
        size_t base = F.cvcw.size();
        F.cvcw.insert(F.cvcw.end(), wt, wt + nv);
        for (int a = c0; a < c1; ++a) {
            int idx = t.wall_cut_index[a];
            if (idx < 0 || idx >= nv) { err = "wall_cut_index out of range"; return KG_ERR_TOPOLOGY; }
            F.cut_idx.push_back(idx); F.cut_gw.push_back(t.wall_cut_gas_w[a]); F.cut_sw.push_back(t.wall_cut_solid_w[a]);
            F.cvcw[base + idx] = 0.0;
        }
        // the donor's neighbour entry for this face must be this wall record
        if (lst(dn, k)[0] != KG_WALL(w)) { err = "donor neighbour entry does not reference its wall record"; return KG_ERR_TOPOLOGY; }
        F.wall_ops.push_back(wo);
    }
    return KG_OK;
}

int flatten(const kg_params& prm, const kg_topology& t, Flat& F, std::string& err) {
    PairIds pid;
    int rc0 = flatten_head(prm, t, F, pid, err);
    if (rc0) return rc0;
    const int D = t.dim, NDF = t.ndf, NC = t.n_cells, NWL = t.n_walls;
    (void)NWL;
    Ctx c{&t, D, NDF, &F, &pid, &err};
    const int NF = 2 * D;
    auto st = [&](int cell, int k) { return (int)t.nbr_state[cell * NF + k]; };
    auto lst = [&](int cell, int k) { return t.nbr_ref + t.nbr_off[cell * NF + k]; };
    auto cnt = [&](int cell, int k) { return (int)(t.nbr_off[cell * NF + k + 1] - t.nbr_off[cell * NF + k]); };
    auto be_of = [&](int data) { return F.dbe[data]; };

    // ---- slope ops (slope!, Flux/Slope.jl:458-1070) ------------------------------------
    const int Lmin = pid.lmin, Lmax = pid.lmax;
    const int half = 1 << (D - 1);
    auto add_list = [&](int cell, int k, int& off, int& n) -> int {
        off = (int)F.slope_nbr.size();
        n = cnt(cell, k);
        for (int j = 0; j < n; ++j) {
            int dn = data_of(c, lst(cell, k)[j]);
            if (dn < 0) { err = "slope list references nothing / inside-solid data"; return KG_ERR_TOPOLOGY; }
            int p = pairing(c, t.cell_grid[cell], F.dgrid[dn]);
            if (p == -2) return KG_ERR_TOPOLOGY;
            F.slope_nbr.push_back(NbrRef{dn, p});
        }
        return KG_OK;
    };
    auto first_data = [&](int cell, int k) { return data_of(c, lst(cell, k)[0]); };
    auto has_offset = [&](int cell, int k) {  // _ps_has_transverse_offset (Slope.jl:177-199)
        int dir = k / 2, n = cnt(cell, k);
        if (n == 0) return false;
        for (int tt = 0; tt < D; ++tt) {
            if (tt == dir) continue;
            double avg = 0.0;
            for (int j = 0; j < n; ++j) avg += dmid(c, data_of(c, lst(cell, k)[j]))[tt];
            avg /= n;
            if (avg != t.cell_midpoint[(size_t)cell * D + tt]) return true;
        }
        return false;
    };
    auto op_one = [&](SlopeOp& op, int cell, int k, double ds, bool proj) -> int {
        op.kind = SLOPE_ONE; op.inv_dsA = 1.0 / ds; op.projA = proj;
        return add_list(cell, k, op.listA, op.cntA);
    };
    auto op_two = [&](SlopeOp& op, int cell, double dsL, double dsR, bool pL, bool pR, int dir) -> int {
        op.kind = SLOPE_TWO; op.inv_dsA = 1.0 / dsL; op.inv_dsB = 1.0 / dsR; op.projA = pL; op.projB = pR;
        int rc = add_list(cell, 2 * dir, op.listA, op.cntA);
        if (rc) return rc;
        return add_list(cell, 2 * dir + 1, op.listB, op.cntB);
    };
    // the neighbour-state dispatcher update_slope!(Val(sL), Val(sR)) (Slope.jl:458-771)
    auto dispatch = [&](SlopeOp& op, int cell, int dir) -> int {
        int kL = 2 * dir, kR = 2 * dir + 1;
        int sL = st(cell, kL), sR = st(cell, kR);
        const double* pm = t.cell_midpoint + (size_t)cell * D;
        double ds = t.cell_ds[(size_t)cell * D + dir];
        if (sL == 1 && sR == 1) {
            bool Ls = be_of(first_data(cell, kL)) < 0, Rs = be_of(first_data(cell, kR)) < 0;
            if (Ls && Rs) { op.kind = SLOPE_ZERO; return KG_OK; }
            if (Ls) return op_one(op, cell, kR, pm[dir] - dmid(c, first_data(cell, kR))[dir], false);
            if (Rs) return op_one(op, cell, kL, pm[dir] - dmid(c, first_data(cell, kL))[dir], false);
            return op_two(op, cell, ds, -ds, false, false, dir);
        }
        if (sL == 0 || sR == 0) {
            if (sL == 0 && sR == 0) { err = "a fluid cell has domain boundaries on both sides of a direction (no reference method)"; return KG_ERR_TOPOLOGY; }
            int k = sL == 0 ? kR : kL;
            return op_one(op, cell, k, pm[dir] - dmid(c, first_data(cell, k))[dir], false);
        }
        auto fac = [&](int s) { return s == 1 ? 1.0 : (s == half ? 0.75 : 1.5); };
        if ((sL != 1 && sL != half && sL != -1) || (sR != 1 && sR != half && sR != -1)) { err = "invalid neighbour state"; return KG_ERR_TOPOLOGY; }
        return op_two(op, cell, fac(sL) * ds, -fac(sR) * ds, false, false, dir);
    };
    // transverse correction (update_slope_transverse_level! step 2, Slope.jl:908-941)
    auto transverse = [&](SlopeOp& op, int cell, int dir) -> int {
        int kL = 2 * dir, kR = 2 * dir + 1;
        int sL = st(cell, kL), sR = st(cell, kR);
        const double* pm = t.cell_midpoint + (size_t)cell * D;
        if (sL != 0 && sR != 0) {
            double dsL = pm[dir] - dmid(c, first_data(cell, kL))[dir];
            double dsR = pm[dir] - dmid(c, first_data(cell, kR))[dir];
            if (be_of(first_data(cell, kL)) < 0) return op_one(op, cell, kR, dsR, true);
            if (be_of(first_data(cell, kR)) < 0) return op_one(op, cell, kL, dsL, true);
            return op_two(op, cell, dsL, dsR, has_offset(cell, kL), has_offset(cell, kR), dir);
        }
        if (sR == 0 && sL == -1) {
            if (be_of(first_data(cell, kL)) < 0) { op.kind = SLOPE_SKIP; return KG_OK; }
            return op_one(op, cell, kL, pm[dir] - dmid(c, first_data(cell, kL))[dir], true);
        }
        if (sL == 0 && sR == -1) {
            if (be_of(first_data(cell, kR)) < 0) { op.kind = SLOPE_SKIP; return KG_OK; }
            return op_one(op, cell, kR, pm[dir] - dmid(c, first_data(cell, kR))[dir], true);
        }
        op.kind = SLOPE_SKIP;
        return KG_OK;
    };
    F.pass_off.push_back(0);
    F.pass_cells_off.push_back(0);
    for (int L = Lmin; L <= Lmax; ++L) {
        for (int i = 0; i < NC; ++i) {
            if (t.cell_bound_enc[i] < 0 || t.cell_level[i] != L) continue;
            F.pass_cells.push_back(i);
            F.cell_slope_op.push_back((int32_t)F.slope_ops.size());
            for (int dir = 0; dir < D; ++dir) {
                SlopeOp op{};
                op.cell = i; op.dir = (int8_t)dir;
                op.kind = SLOPE_SKIP;
                int sL = st(i, 2 * dir), sR = st(i, 2 * dir + 1);
                int rc;
                if (L == Lmin || !(sL == -1 || sR == -1)) rc = dispatch(op, i, dir);
                else rc = transverse(op, i, dir);
                if (rc) return rc;
                F.slope_ops.push_back(op);
            }
            int nlist = 0;
            for (int dir = 0; dir < D; ++dir) {
                const SlopeOp& o = F.slope_ops[F.slope_ops.size() - D + dir];
                if (o.kind == SLOPE_ONE || o.kind == SLOPE_TWO) nlist += o.cntA;
                if (o.kind == SLOPE_TWO) nlist += o.cntB;
            }
            if (nlist > 2 * MAXD * 4) { err = "a cell's slope neighbour lists exceed 24 entries (not 2:1 balanced)"; return KG_ERR_TOPOLOGY; }
        }
        F.pass_off.push_back((int32_t)F.slope_ops.size());
        F.pass_cells_off.push_back((int32_t)F.pass_cells.size());
    }
    // The passes by dependency depth instead of by level: only a transverse projection reads
    // other cells' slopes of this step (those of its coarser neighbours, computed by an earlier
    // pass of the level sweep, Slope.jl:908-941); every other cell reads f alone and joins the
    // first pass.  A cell's pass follows the passes of the cells whose slopes it reads, so every
    // cell computes the same values as in the level order, in fewer, fuller launches.
    {
        const size_t npc = F.pass_cells.size();
        std::vector<int32_t> entry((size_t)NC, -1), depth(npc, 0);
        for (size_t k = 0; k < npc; ++k) entry[F.pass_cells[k]] = (int32_t)k;
        bool ok = true;
        int maxd = 0;
        for (size_t k = 0; k < npc && ok; ++k) {
            int dk = 0;
            for (int dir = 0; dir < D; ++dir) {
                const SlopeOp& op = F.slope_ops[(size_t)F.cell_slope_op[k] + dir];
                if (op.kind != SLOPE_ONE && op.kind != SLOPE_TWO) continue;
                for (int side = 0; side < 2; ++side) {
                    const bool proj = side == 0 ? op.projA : (op.kind == SLOPE_TWO && op.projB);
                    if (!proj) continue;
                    const int32_t l0 = side == 0 ? op.listA : op.listB, n = side == 0 ? op.cntA : op.cntB;
                    for (int32_t j = 0; j < n; ++j) {
                        const int32_t dn = F.slope_nbr[(size_t)l0 + j].data;
                        if (dn >= NC || entry[dn] < 0) continue;   // walls, solid cells: no slope pass
                        if ((size_t)entry[dn] >= k) { ok = false; break; }   // not coarser: keep the level passes
                        dk = std::max(dk, depth[entry[dn]] + 1);
                    }
                }
            }
            depth[k] = dk;
            maxd = std::max(maxd, dk);
        }
        if (ok) {
            std::vector<int32_t> cells, ops;
            cells.reserve(npc);
            ops.reserve(npc);
            F.pass_cells_off.assign(1, 0);
            for (int d = 0; d <= maxd; ++d) {
                for (size_t k = 0; k < npc; ++k)
                    if (depth[k] == d) { cells.push_back(F.pass_cells[k]); ops.push_back(F.cell_slope_op[k]); }
                F.pass_cells_off.push_back((int32_t)cells.size());
            }
            F.pass_cells.swap(cells);
            F.cell_slope_op.swap(ops);
        }
    }

    // ---- physical-space criterion (update_criterion!, Physical_space/AMR.jl:1-284) --------
    for (int i = 0; i < NC; ++i) {
        if (t.cell_bound_enc[i] < 0) continue;
        for (int dir = 0; dir < D; ++dir) {
            CritOp op{};
            const int sA = st(i, 2 * dir), sB = st(i, 2 * dir + 1);
            const double ds = t.cell_ds[(size_t)i * D + dir];
            auto factor = [&](int s) { return s == 1 ? 1.0 : (s == -1 ? 1.5 : 0.75); };
            auto add = [&](int k, int32_t* lst0, int32_t* n) {
                *lst0 = (int32_t)F.crit_nbr.size();
                *n = cnt(i, k);
                for (int j = 0; j < *n; ++j) {
                    const int32_t r = lst(i, k)[j];
                    F.crit_nbr.push_back(r >= 0 ? r : -1);   // -1: a SolidNeighbor (w = sw = 0)
                }
            };
            // the lists of every non-boundary side (the buffer layer of apply_amr_buffer! reads
            // them even when the other side is a boundary)
            if (sA != 0) add(2 * dir, &op.listA, &op.cntA);
            if (sB != 0) add(2 * dir + 1, &op.listB, &op.cntB);
            op.dsA = factor(sA) * ds;
            op.dsB = factor(sB) * ds;
            op.coarseA = sA == -1;
            op.coarseB = sB == -1;
            op.kind = (sA != 0 && sB != 0) ? 1 : 0;
            F.crit_ops.push_back(op);
        }
    }

    // ---- flux incidences (flux!, Flux/Flux.jl:19-111,458-503) -----------------------------
    // Per cell its incidences in face order, in one array: count them, then place them.
    std::vector<int32_t> nper(NC + 1, 0);
    for (int fi = 0; fi < t.n_faces; ++fi) {
        const int here = t.face_here[fi];
        if (here < 0 || here >= NC) { err = "face here side must be a fluid cell"; return KG_ERR_TOPOLOGY; }
        nper[here + 1] += 1;
        if (t.face_kind[fi] != KG_FACE_DOMAIN) {
            const int od = data_ref(t, t.face_there[fi]);
            if (od >= 0 && od < NC && F.dbe[od] >= 0) nper[od + 1] += 1;
        }
    }
    for (int i = 0; i < NC; ++i) nper[i + 1] += nper[i];
    F.inc.resize((size_t)nper[NC]);
    Incidence* incs = F.inc.data();
    std::vector<int32_t> fill(nper.begin(), nper.end() - 1);
    for (int fi = 0; fi < t.n_faces; ++fi) {
        Incidence a{};
        int dir = t.face_dir[fi];
        if (dir < 0 || dir >= D) { err = "face_dir out of range"; return KG_ERR_TOPOLOGY; }
        int here = t.face_here[fi];
        if (here < 0 || here >= NC || t.cell_bound_enc[here] < 0) { err = "face here side must be a fluid cell"; return KG_ERR_TOPOLOGY; }
        double rot = t.face_rot[fi], area = t.face_area[fi];
        if (rot != 1.0 && rot != -1.0) { err = "face_rot must be +1 or -1"; return KG_ERR_TOPOLOGY; }
        for (int d = 0; d < D; ++d) { a.fmid[d] = t.face_midpoint[(size_t)fi * D + d]; a.my_mid[d] = t.cell_midpoint[(size_t)here * D + d]; }
        a.dir = (int8_t)dir;
        if (t.face_kind[fi] == KG_FACE_DOMAIN) {
            int bk = t.face_bc_kind[fi];
            if (bk < KG_BC_MAXWELL || bk > KG_BC_INTERP) { err = "unknown domain boundary kind"; return KG_ERR_TOPOLOGY; }
            if (bk == KG_BC_MAXWELL && prm.flux == KG_FLUX_DVM) { err = "DVM Maxwellian domain flux is undefined in the reference (DVM.jl:3,12)"; return KG_ERR_TOPOLOGY; }
            if (bk == KG_BC_INTERP && D != 2) { err = "InterpolatedOutflow is 2D only in the reference"; return KG_ERR_TOPOLOGY; }
            a.kind = INC_DOMAIN; a.bc_kind = (int8_t)bk; a.other = -1; a.pair = -1; a.here_side = 1;
            a.orient = rot; a.sarea = area;
            a.bc = (int32_t)(F.bc_prim.size() / MAXW);
            for (int e = 0; e < MAXW; ++e) F.bc_prim.push_back(e < D + 2 ? t.face_bc[(size_t)fi * (D + 2) + e] : 0.0);
            {
                const double* b = &F.bc_prim[F.bc_prim.size() - MAXW];
                for (int e = 0; e < MAXW; ++e) F.bc_hl.push_back((float)b[e]);
                for (int e = 0; e < MAXW; ++e) F.bc_hl.push_back((float)(b[e] - (double)(float)b[e]));
            }
            incs[fill[here]++] = a;
            continue;
        }
        int od = data_ref(t, t.face_there[fi]);
        if (od < 0) { err = "inner face without a there side"; return KG_ERR_TOPOLOGY; }
        bool solid = F.dbe[od] < 0;
        a.kind = solid ? INC_SOLID : INC_INNER;
        a.other = od; a.here_side = 1; a.orient = rot; a.sarea = area;
        for (int d = 0; d < D; ++d) { a.ot_mid[d] = t.face_there_midpoint[(size_t)fi * D + d]; a.ot_ds[d] = F.dds[(size_t)od * MAXD + d]; }
        a.pair = pairing(c, t.cell_grid[here], F.dgrid[od]);
        if (a.pair == -2) return KG_ERR_TOPOLOGY;
        if (solid && od >= NC && F.dgrid[od] != t.cell_grid[here]) { err = "wall grid differs from donor grid"; return KG_ERR_TOPOLOGY; }
        if (solid && od >= NC) {
            a.wallrec = 1;
            a.pert = a.ot_mid[dir] - t.wall_aux_point[(size_t)(od - NC) * D + dir];
        }
        incs[fill[here]++] = a;
        if (!solid && od < NC) {
            // the there side receives the same flux with the opposite sign
            Incidence b{};
            b.kind = INC_INNER; b.dir = (int8_t)dir; b.other = here; b.here_side = 0;
            b.orient = -rot; b.sarea = -area;
            for (int d = 0; d < D; ++d) {
                b.fmid[d] = a.fmid[d];
                b.my_mid[d] = a.ot_mid[d];                // the (possibly periodic-shifted) copy
                b.ot_mid[d] = a.my_mid[d];
                b.ot_ds[d] = t.cell_ds[(size_t)here * D + d];
            }
            b.pair = pairing(c, t.cell_grid[od], t.cell_grid[here]);
            if (b.pair == -2) return KG_ERR_TOPOLOGY;
            incs[fill[od]++] = b;
        }
    }
    // cells with bound_enc < 0 hold no incidences (a face's here side is fluid, and only a
    // fluid there side is updated), so the per-cell runs in cell order are the fluid list's
    F.inc_off.push_back(0);
    for (int i = 0; i < NC; ++i) {
        if (t.cell_bound_enc[i] < 0) continue;
        F.fluid_cells.push_back(i);
        int nbcm = 0;
        const Incidence* pi = F.inc.data() + nper[i];
        const int ni = nper[i + 1] - nper[i];
        for (int q = 0; q < ni; ++q) {
            const Incidence& a = pi[q];
            if (a.kind == INC_DOMAIN && (a.bc_kind == KG_BC_MAXWELL || a.bc_kind == KG_BC_INFLOW)) ++nbcm;
        }
        F.max_inc = std::max(F.max_inc, ni);
        F.max_bcm = std::max(F.max_bcm, nbcm);
        // regular cell: per direction one face at -ds/2 and one at +ds/2, each an inner face to
        // a same-sized fluid neighbour on this cell's velocity grid, oriented so that a velocity
        // leaves through the face it points at (the flux kernel's fast path relies on all of it)
        bool reg = ni == 2 * D;
        int seen[2 * MAXD] = {0};
        for (int q = 0; q < ni; ++q) {
            const Incidence& a = pi[q];
            if (!reg) break;
            const int d = a.dir;
            const double h = 0.5 * t.cell_ds[(size_t)i * D + d];
            const double dm = a.fmid[d] - a.my_mid[d], dox = a.fmid[d] - a.ot_mid[d];
            reg = a.kind == INC_INNER && a.pair < 0 && a.other >= 0 && a.other < NC &&
                  std::fabs(std::fabs(dm) - h) <= 1e-12 * h && std::fabs(dox + dm) <= 1e-12 * h &&
                  a.orient * dm < 0.0;
            for (int e = 0; reg && e < D; ++e) {
                if (e != d && (std::fabs(a.fmid[e] - a.my_mid[e]) > 1e-12 * h || std::fabs(a.fmid[e] - a.ot_mid[e]) > 1e-12 * h)) reg = false;
                if (a.ot_ds[e] != t.cell_ds[(size_t)i * D + e]) reg = false;
            }
            if (reg) ++seen[2 * d + (dm > 0.0 ? 1 : 0)];
        }
        for (int e = 0; reg && e < 2 * D; ++e) reg = seen[e] == 1;
        F.fluid_reg.push_back(reg ? 1 : 0);
        F.inc_off.push_back(nper[i + 1]);
    }

    {
        const int rc = flatten_ib(t, F, pid, err);
        if (rc) return rc;
    }
    if (F.p_j0.empty()) { F.p_j0.push_back(0); F.p_cnt.push_back(0); }
    return KG_OK;
}

void merge(const std::vector<Part>& parts, int32_t dcap, Flat& M, std::vector<int32_t>& ranges, bool fuse, bool light) {
    reset(M);
    if (parts.empty()) return;
    const int D = parts[0].F->dim;
    M.dim = D; M.ndf = parts[0].F->ndf;
    M.n_data = dcap;
    int64_t PGtot = 0;
    for (auto& p : parts) PGtot += (int64_t)p.F->vw.size();
    M.vu.assign((size_t)D * PGtot, 0.0);
    M.vuf.assign((size_t)D * PGtot, 0.0f);
    M.vidx.assign((size_t)D * PGtot, 0);
    M.g_off.push_back(0);
    M.p_off.push_back(0);
    M.foff.assign((size_t)dcap + 1, 0);
    M.dgrid.assign(dcap, 0); M.dbe.assign(dcap, 0); M.dnv.assign(dcap, 0); M.dprob.assign(dcap, -1);
    M.dinvv.assign(dcap, 0.0);
    M.dmid.assign((size_t)dcap * MAXD, 0.0); M.dds.assign((size_t)dcap * MAXD, 0.0);
    M.inc_off.push_back(0);
    {
        size_t ninc = 0, nfl = 0, nso = 0, nsn = 0, np = 0, npo = 0, nco = 0, ncn = 0;
        for (auto& p : parts) {
            ninc += p.F->inc.size(); nfl += p.F->fluid_cells.size(); nso += p.F->slope_ops.size();
            nsn += p.F->slope_nbr.size(); np += p.F->p_j0.size(); npo += p.F->p_off.size();
            nco += p.F->crit_ops.size(); ncn += p.F->crit_nbr.size();
        }
        M.inc.reserve(ninc); M.fcrec.reserve(nfl); M.regrec.reserve(nfl); M.fluid_cells.reserve(nfl); M.fluid_reg.reserve(nfl);
        M.inc_off.reserve(nfl + 1); M.slope_ops.reserve(nso); M.slope_nbr.reserve(nsn);
        M.p_j0.reserve(np); M.p_cnt.reserve(np); M.p_off.reserve(npo + 1);
        M.crit_ops.reserve(nco); M.crit_nbr.reserve(ncn);
    }
    size_t npass = 0;
    for (auto& p : parts) npass = std::max(npass, p.F->pass_cells_off.size() - 1);
    int64_t PGacc = 0;
    int32_t Gacc = 0;
    ranges.clear();
    for (auto& p : parts) {
        const Flat& F = *p.F;
        const int64_t PG = (int64_t)F.vw.size();
        const int32_t G = (int32_t)F.g_off.size() - 1;
        const int32_t pairacc = (int32_t)M.p_off.size() - 1;
        const int64_t ptab = (int64_t)M.p_j0.size();
        const int32_t snb = (int32_t)M.slope_nbr.size();
        const int32_t sops = (int32_t)M.slope_ops.size();
        const int32_t incacc = (int32_t)M.inc.size();
        const int32_t bcacc = (int32_t)(M.bc_prim.size() / MAXW);
        const int32_t ibacc = (int32_t)M.ib_nbr.size();
        const int32_t cutacc = (int32_t)M.cut_idx.size();
        const int64_t cvacc = (int64_t)M.cvcw.size();
        const int32_t axacc = (int32_t)M.ax_val.size();
        // velocity grids
        for (int g = 0; g < G; ++g) M.g_off.push_back(PGacc + F.g_off[g + 1]);
        M.vlev.insert(M.vlev.end(), F.vlev.begin(), F.vlev.end());
        M.vw.insert(M.vw.end(), F.vw.begin(), F.vw.end());
        M.vwf.insert(M.vwf.end(), F.vwf.begin(), F.vwf.end());
        for (int d = 0; d < D; ++d)
            for (int64_t i = 0; i < PG; ++i) {
                M.vu[(size_t)d * PGtot + PGacc + i] = F.vu[(size_t)d * PG + i];
                M.vuf[(size_t)d * PGtot + PGacc + i] = F.vuf[(size_t)d * PG + i];
                M.vidx[(size_t)d * PGtot + PGacc + i] = F.vidx[(size_t)d * PG + i];
            }
        for (int g = 0; g < G; ++g)
            for (int d = 0; d < MAXD; ++d) M.ax_off.push_back(axacc + F.ax_off[(size_t)g * MAXD + d]);
        M.ax_val.insert(M.ax_val.end(), F.ax_val.begin(), F.ax_val.end());
        M.ax_hi.insert(M.ax_hi.end(), F.ax_hi.begin(), F.ax_hi.end());
        M.ax_lo.insert(M.ax_lo.end(), F.ax_lo.begin(), F.ax_lo.end());
        M.max_axis = std::max(M.max_axis, F.max_axis);
        M.max_nv = std::max(M.max_nv, F.max_nv);
        M.max_inc = std::max(M.max_inc, F.max_inc);
        M.max_bcm = std::max(M.max_bcm, F.max_bcm);
        M.phase_cells += F.phase_cells;
        M.n_cells += F.n_cells;
        M.n_walls += F.n_walls;
        // data table at pool positions
        for (int j = 0; j < F.n_data; ++j) {
            const int32_t m = p.dbase + j;
            M.foff[m] = p.fbase + F.foff[j];
            M.dgrid[m] = Gacc + F.dgrid[j];
            M.dbe[m] = F.dbe[j];
            M.dnv[m] = F.dnv[j];
            M.dprob[m] = p.slot;
            M.dinvv[m] = F.dinvv[j];
            for (int d = 0; d < MAXD; ++d) { M.dmid[(size_t)m * MAXD + d] = F.dmid[(size_t)j * MAXD + d]; M.dds[(size_t)m * MAXD + d] = F.dds[(size_t)j * MAXD + d]; }
        }
        // pairings
        for (size_t q = 1; q < F.p_off.size(); ++q) M.p_off.push_back(ptab + F.p_off[q]);
        if (F.p_off.size() > 1) {
            M.p_j0.insert(M.p_j0.end(), F.p_j0.begin(), F.p_j0.begin() + F.p_off.back());
            M.p_cnt.insert(M.p_cnt.end(), F.p_cnt.begin(), F.p_cnt.begin() + F.p_off.back());
        }
        auto rp = [&](int32_t pr) { return pr >= 0 ? pr + pairacc : pr; };
        int32_t fb = (int32_t)M.fluid_cells.size();
        for (int c : F.fluid_cells) M.fluid_cells.push_back(c + p.dbase);
        M.fluid_reg.insert(M.fluid_reg.end(), F.fluid_reg.begin(), F.fluid_reg.end());
        if (!light) {
        // slope ops and neighbour lists
        for (SlopeOp op : F.slope_ops) { op.cell += p.dbase; op.listA += snb; op.listB += snb; M.slope_ops.push_back(op); }
        for (NbrRef r : F.slope_nbr) { r.data += p.dbase; r.pair = rp(r.pair); M.slope_nbr.push_back(r); }
        // flux incidences
        for (size_t q = 1; q < F.inc_off.size(); ++q) M.inc_off.push_back(incacc + F.inc_off[q]);
        for (Incidence a : F.inc) {
            if (a.other >= 0) {
                a.other += p.dbase;
                a.ofoff = M.foff[a.other];
                a.onv = M.dnv[a.other];
                a.ogo = (int32_t)M.g_off[M.dgrid[a.other]];
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
            a.pair = rp(a.pair);
            a.bc += bcacc;
            M.inc.push_back(a);
        }
        for (size_t k = 0; k < F.fluid_cells.size(); ++k) {
            const int32_t m = F.fluid_cells[k] + p.dbase;
            FluxCell fc{};
            fc.foff = M.foff[m];
            fc.goff = M.g_off[M.dgrid[m]];
            fc.invV = M.dinvv[m];
            for (int d = 0; d < MAXD; ++d) fc.ds[d] = M.dds[(size_t)m * MAXD + d];
            fc.cell = m; fc.slot = p.slot;
            fc.inc0 = incacc + F.inc_off[k];
            fc.ninc = F.inc_off[k + 1] - F.inc_off[k];
            fc.nv = M.dnv[m]; fc.gid = M.dgrid[m]; fc.reg = F.fluid_reg[k];
            M.fcrec.push_back(fc);
            RegRec rr{};
            if (fc.reg) {
                for (int q = 0; q < fc.ninc; ++q) {
                    const Incidence& a = M.inc[(size_t)fc.inc0 + q];
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
            M.regrec.push_back(rr);
        }
        {
            const int32_t cacc = (int32_t)M.crit_nbr.size();
            for (CritOp op : F.crit_ops) { op.listA += cacc; op.listB += cacc; M.crit_ops.push_back(op); }
            for (int32_t r : F.crit_nbr) M.crit_nbr.push_back(r >= 0 ? r + p.dbase : -1);
        }
        M.bc_prim.insert(M.bc_prim.end(), F.bc_prim.begin(), F.bc_prim.end());
        M.bc_hl.insert(M.bc_hl.end(), F.bc_hl.begin(), F.bc_hl.end());
        }   // !light
        ranges.push_back(fb);
        ranges.push_back((int32_t)M.fluid_cells.size());
        M.n_fluid += F.n_fluid;
        // immersed boundary
        for (SolidOp so : F.solid_ops) { so.cell += p.dbase; so.list += ibacc; M.solid_ops.push_back(so); }
        for (WallOp wo : F.wall_ops) {
            wo.donor += p.dbase; wo.solid += p.dbase; wo.data += p.dbase; wo.list += ibacc;
            wo.spair = rp(wo.spair); wo.cut_off += cutacc; wo.cvcw_off += cvacc;
            M.wall_ops.push_back(wo);
        }
        for (NbrRef r : F.ib_nbr) { r.data += p.dbase; r.pair = rp(r.pair); M.ib_nbr.push_back(r); }
        M.ib_dx.insert(M.ib_dx.end(), F.ib_dx.begin(), F.ib_dx.end());
        M.cut_idx.insert(M.cut_idx.end(), F.cut_idx.begin(), F.cut_idx.end());
        M.cut_gw.insert(M.cut_gw.end(), F.cut_gw.begin(), F.cut_gw.end());
        M.cut_sw.insert(M.cut_sw.end(), F.cut_sw.begin(), F.cut_sw.end());
        M.cvcw.insert(M.cvcw.end(), F.cvcw.begin(), F.cvcw.end());
        PGacc += PG;
        Gacc += G;
        (void)sops;
    }
    M.ax_off.push_back((int32_t)M.ax_val.size());
    // slope passes merged by their index relative to each problem's coarsest level
    M.pass_off.push_back(0);
    M.pass_cells_off.push_back(0);
    std::vector<int32_t> sops_base;
    {
        int32_t acc = 0;
        for (auto& p : parts) { sops_base.push_back(acc); acc += (int32_t)p.F->slope_ops.size(); }
    }
    for (size_t ps = 0; ps < npass; ++ps) {
        for (size_t q = 0; q < parts.size(); ++q) {
            const Flat& F = *parts[q].F;
            if (ps + 1 >= F.pass_cells_off.size()) continue;
            for (int32_t k = F.pass_cells_off[ps]; k < F.pass_cells_off[ps + 1]; ++k) {
                M.pass_cells.push_back(F.pass_cells[k] + parts[q].dbase);
                if (!light) M.cell_slope_op.push_back(F.cell_slope_op[k] + sops_base[q]);
            }
        }
        M.pass_off.push_back((int32_t)M.slope_ops.size());
        M.pass_cells_off.push_back((int32_t)M.pass_cells.size());
    }
    if (light) return;
    M.screc.resize(M.pass_cells.size());
    for (size_t k = 0; k < M.pass_cells.size(); ++k) {
        const int32_t m = M.pass_cells[k];
        SlopeCell c{};
        c.foff = M.foff[m];
        c.nv = M.dnv[m];
        bool reg = true;
        for (int d = 0; d < D && reg; ++d) {
            const SlopeOp& op = M.slope_ops[M.cell_slope_op[k] + d];
            reg = op.kind == SLOPE_TWO && op.cntA == 1 && op.cntB == 1 && !op.projA && !op.projB;
            if (!reg) break;
            const NbrRef a = M.slope_nbr[op.listA], b = M.slope_nbr[op.listB];
            reg = a.pair < 0 && b.pair < 0 && M.dnv[a.data] == c.nv && M.dnv[b.data] == c.nv;
            c.nfoff[2 * d] = M.foff[a.data];
            c.nfoff[2 * d + 1] = M.foff[b.data];
            c.inv_d[2 * d] = op.inv_dsA;
            c.inv_d[2 * d + 1] = op.inv_dsB;
            c.inv_f[2 * d] = (float)op.inv_dsA;
            c.inv_f[2 * d + 1] = (float)op.inv_dsB;
        }
        c.regular = reg ? 1 : 0;
        M.screc[k] = c;
    }
    // Slopes in the flux kernel (fuse: 2D layouts of the packed regular-cell kernel).  A
    // regular cell whose own slopes and whose four neighbours' slopes are of the regular form
    // (slope-regular, and the neighbours flux-regular: fluid cells on the same grid whose f
    // nothing writes during a step) gets an R2Rec; one whose four neighbours all have one reads
    // no sdf and no other cell reads its sdf in a step, so its slopes leave the passes (lazy
    // items, computed only where a sync point reads the slopes).
    M.fluid_r2.assign((size_t)M.n_fluid, 0);
    M.r2rec.assign((size_t)M.n_fluid, R2Rec{});
    if (fuse && D == 2) {
        std::vector<int32_t> dsc((size_t)dcap, -1), dfl((size_t)dcap, -1);
        for (size_t k = 0; k < M.pass_cells.size(); ++k) dsc[M.pass_cells[k]] = (int32_t)k;
        for (int q = 0; q < M.n_fluid; ++q) dfl[M.fluid_cells[q]] = q;
        auto slope_reg = [&](int32_t m) { return m >= 0 && m < dcap && dsc[m] >= 0 && M.screc[dsc[m]].regular; };
        for (int q = 0; q < M.n_fluid; ++q) {
            const int32_t m = M.fluid_cells[q];
            if (!M.fluid_reg[q] || !slope_reg(m)) continue;
            const RegRec& rr = M.regrec[q];
            const SlopeCell& me = M.screc[dsc[m]];
            bool ok = true;
            for (int sd = 0; sd < 4 && ok; ++sd) {
                const int32_t n = rr.nd[sd];
                ok = n >= 0 && n < dcap && dfl[n] >= 0 && M.fluid_reg[dfl[n]] && slope_reg(n) && me.nfoff[sd] == rr.nfo[sd];
            }
            if (!ok) continue;
            R2Rec r{};
            for (int t = 0; t < 4; ++t) r.sinv[t] = me.inv_f[t];
            for (int sd = 0; sd < 4; ++sd) {
                const SlopeCell& nb = M.screc[dsc[rr.nd[sd]]];
                for (int t = 0; t < 4; ++t) { r.nn[sd][t] = nb.nfoff[t]; r.ninv[sd][t] = nb.inv_f[t]; }
            }
            M.r2rec[q] = r;
            M.fluid_r2[q] = 1;
        }
        for (int q = 0; q < M.n_fluid; ++q) {
            if (!M.fluid_r2[q]) continue;
            bool interior = true;
            for (int sd = 0; sd < 4 && interior; ++sd) interior = M.fluid_r2[dfl[M.regrec[q].nd[sd]]] != 0;
            if (interior) M.fluid_r2[q] = 2;
        }
    }
    slope_items(M, dcap, fuse);
}

void slope_items(Flat& M, int32_t dcap, bool fuse) {
    const int D = M.dim;
    M.slope_items.clear();
    M.pass_items_off.clear();
    // work items of the slope passes: when some grid exceeds two chunks, a pass cell per
    // SLOPE_CHUNK velocity cells (large 3D grids: fewer cells than resident CTAs per level);
    // otherwise one item per pass cell (the kernel indexes the pass cells directly when every
    // pass cell has its item in order, i.e. without lazy items)
    bool split = false;
    for (int32_t m : M.pass_cells) split |= M.dnv[m] > 2 * SLOPE_CHUNK;
    std::vector<uint8_t> lazy(M.pass_cells.size(), 0);
    if (fuse && D == 2) {
        std::vector<int32_t> dfl((size_t)dcap, -1);
        for (int q = 0; q < M.n_fluid; ++q) dfl[M.fluid_cells[q]] = q;
        for (size_t k = 0; k < M.pass_cells.size(); ++k) {
            const int32_t q = dfl[M.pass_cells[k]];
            lazy[k] = q >= 0 && M.fluid_r2[q] == 2;
        }
    }
    M.pass_items_off.push_back(0);
    for (size_t ps = 0; ps + 1 < M.pass_cells_off.size(); ++ps) {
        for (int32_t k = M.pass_cells_off[ps]; k < M.pass_cells_off[ps + 1]; ++k) {
            if (lazy[k]) continue;
            const int nch = split ? (M.dnv[M.pass_cells[k]] + SLOPE_CHUNK - 1) / SLOPE_CHUNK : 1;
            for (int c = 0; c < nch; ++c) { M.slope_items.push_back(k); M.slope_items.push_back(c); }
        }
        M.pass_items_off.push_back((int32_t)(M.slope_items.size() / 2));
    }
    for (size_t k = 0; k < M.pass_cells.size(); ++k) {
        if (!lazy[k]) continue;
        const int nch = split ? (M.dnv[M.pass_cells[k]] + SLOPE_CHUNK - 1) / SLOPE_CHUNK : 1;
        for (int c = 0; c < nch; ++c) { M.slope_items.push_back((int32_t)k); M.slope_items.push_back(c); }
    }
    M.pass_items_off.push_back((int32_t)(M.slope_items.size() / 2));
    if (M.p_j0.empty()) { M.p_j0.push_back(0); M.p_cnt.push_back(0); }
}

int64_t device_bytes(const Flat& F, int precision) {
    int64_t s = precision == KG_PREC_FP64 ? 8 : 4;
    int64_t nf = F.foff.back();
    int64_t b = 0;
    b += 2 * nf * s;                       // f ping-pong
    b += nf * F.dim * s;                   // sdf
    b += (int64_t)F.n_data * (MAXW * 8) * 3;  // w, prim, qf
    b += (int64_t)F.vu.size() * 8 + (int64_t)F.vw.size() * 8 + (int64_t)F.vlev.size();
    b += (int64_t)(F.p_j0.size() + F.p_cnt.size()) * 4;
    b += (int64_t)F.slope_ops.size() * sizeof(SlopeOp) + (int64_t)F.slope_nbr.size() * sizeof(NbrRef);
    b += (int64_t)F.inc.size() * sizeof(Incidence) + (int64_t)F.fluid_cells.size() * sizeof(FluxCell);
    b += (int64_t)F.wall_ops.size() * sizeof(WallOp) + (int64_t)F.cvcw.size() * 8;
    b += (int64_t)F.n_data * 64;
    return b;
}

}  // namespace kg

namespace kg {

// Leaves are keyed by (level, index of their lower corner at that level); the leaf containing
// a finest-level point is the key found first from the finest level down.  The corner and the
// probe are computed with the reference's arithmetic (round of the corner, floor of the probe
// across the face at the face-centre line), so the answers are the leaves its sorted-key search
// returns.
void vs_face_table(const Flat& M, const double* vmin, const double* hf, const int32_t* trees, int maxlevel,
                   std::vector<int32_t>& nbr) {
    const int D = M.dim;
    const int64_t PG = (int64_t)M.vw.size();
    nbr.assign((size_t)PG * 2 * D, -1);
    const int G = (int)M.g_off.size() - 1;
    std::unordered_map<uint64_t, int32_t> leaf;
    auto key = [&](int L, const int64_t* g) {
        uint64_t k = (uint64_t)L;
        for (int d = 0; d < D; ++d) k = (k << 20) | (uint64_t)(g[d] >> (maxlevel - L));
        return k;
    };
    for (int gi = 0; gi < G; ++gi) {
        const int64_t o = M.g_off[gi], nv = M.g_off[gi + 1] - o;
        leaf.clear();
        leaf.reserve((size_t)nv * 2);
        for (int64_t i = 0; i < nv; ++i) {
            const int L = M.vlev[o + i];
            int64_t g[MAXD];
            for (int d = 0; d < D; ++d) {
                const double cell = hf[d] * (double)(1L << (maxlevel - L));
                g[d] = (int64_t)std::nearbyint((M.vu[(size_t)d * PG + o + i] - 0.5 * cell - vmin[d]) / hf[d]);
            }
            leaf[key(L, g)] = (int32_t)i;
        }
        for (int64_t i = 0; i < nv; ++i) {
            const int L = M.vlev[o + i];
            for (int dim = 0; dim < D; ++dim) {
                for (int side = 0; side < 2; ++side) {
                    const int dir = side == 0 ? -1 : 1;
                    const double cell = hf[dim] * (double)(1L << (maxlevel - L));
                    int64_t g[MAXD];
                    bool inside = true;
                    for (int d = 0; d < D && inside; ++d) {
                        double coord = M.vu[(size_t)d * PG + o + i];
                        if (d == dim) coord += dir * (0.5 * cell + 0.5 * hf[d]);
                        g[d] = (int64_t)std::floor((coord - vmin[d]) / hf[d]);
                        inside = g[d] >= 0 && g[d] < ((int64_t)trees[d] << maxlevel);
                    }
                    if (!inside) continue;
                    for (int l = maxlevel; l >= 0; --l) {
                        auto it = leaf.find(key(l, g));
                        if (it != leaf.end()) { nbr[(size_t)(o + i) * 2 * D + 2 * dim + side] = it->second; break; }
                    }
                }
            }
        }
    }
}

}  // namespace kg
