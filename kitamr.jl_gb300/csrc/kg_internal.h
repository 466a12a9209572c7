// kg_internal.h -- device-side layout of libkitgpu.so.
//
// The reference-shaped kg_topology (scatter form: a face list whose faces update
// both adjacent cells) is flattened on the host into a gather form: every cell
// owns the list of (sub-)faces it receives fluxes through ("incidences"), its
// slope operations per direction, and the velocity pairing tables that replace
// the reference's level merge walks.  Each cell is then advanced by one CTA that
// writes only its own data, so no atomics are needed and results are
// deterministic.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>
#include "../../include/kitgpu.h"

namespace kg {

constexpr int MAXD = 3;
constexpr int MAXW = MAXD + 2;
// velocity cells of one slope work item: a multiple of the cells a CTA covers per pass (two
// per thread at 128 or 256 threads), so a large grid spreads over several CTAs
constexpr int SLOPE_CHUNK = 4096;

// ---- slope operations (one per fluid cell and direction) -------------------
enum SlopeKind : int8_t { SLOPE_ZERO = 0, SLOPE_SKIP = 1, SLOPE_ONE = 2, SLOPE_TWO = 3 };

struct SlopeOp {            // 48 bytes
    double inv_dsA, inv_dsB;   // 1/ds of list A, list B
    int32_t listA, cntA;       // into slope_nbr
    int32_t listB, cntB;
    int8_t kind, projA, projB, dir;
    int32_t cell;
};

// update_criterion! of one fluid cell and direction (Physical_space/AMR.jl:1-253): the
// neighbour lists of both sides (-1: a SolidNeighbor, whose w and sw are zeros), their
// distances (ds, 0.75 ds for finer, 1.5 ds for a coarser side) and whether a side is coarser
// (transverse correction from its first neighbour).  kind 0: a domain-boundary side, the
// row is zero.
struct CritOp {
    double dsA, dsB;
    int32_t listA, cntA, listB, cntB;   // into crit_nbr (data indices)
    int8_t kind, coarseA, coarseB, pad;
    int32_t pad2;
};

// A pass-cell entry of the slope sweep in one record (built when the problems are merged).
// Regular: every direction takes a two-sided slope from one neighbour per side, on the
// cell's own velocity grid and without transverse projection; the kernel then needs
// nothing else (the generic path reads the SlopeOps and their neighbour lists).
struct SlopeCell {
    int64_t foff;                 // f offset of the cell
    int64_t nfoff[2 * MAXD];      // f offsets of the neighbours: per direction side A, side B
    double inv_d[2 * MAXD];       // 1/ds of those sides
    float inv_f[2 * MAXD];
    int32_t nv, regular;
};

struct NbrRef {             // neighbour in a slope / extrapolation list
    int32_t data;           // data index (cell, or n_cells + wall)
    int32_t pair;           // velocity pairing id (my grid <- its grid), -1 = identity
};

// ---- flux incidences ------------------------------------------------------
enum IncKind : int8_t { INC_INNER = 0, INC_DOMAIN = 1, INC_SOLID = 2 };
// INC_SOLID: the across-face data has bound_enc < 0 (SolidNeighbor wall record or a
// solid PsData); the reference reconstructs the here side without the positivity
// limiter and (CAIDVM) takes the there side unreconstructed.

struct Incidence {          // 208 bytes
    double fmid[MAXD];      // face (sub-face) midpoint
    double my_mid[MAXD];    // centre used for this cell's reconstruction
    double ot_mid[MAXD];    // centre used for the other side's reconstruction
    double orient;          // +rot if this cell is the face's here side, -rot otherwise
    double sarea;           // +area (here) / -area (there): factor of the received flux
    double ot_ds[MAXD];     // other side's ds (positivity limiter)
    int32_t other;          // data index of the other side (-1 for a domain face)
    int32_t pair;           // pairing (my grid <- other's grid), -1 identity
    int8_t kind, dir, bc_kind, here_side;
    int32_t bc;             // index into bc_prim (domain faces)
    // resolved when the problems are merged, so the flux kernel needs no further lookups:
    int64_t ofoff;          // f offset of the other side (-1 for a domain face)
    int32_t onv, ogo;       // its velocity count and grid offset
    float dxm_f[MAXD], dxo_f[MAXD], ods_f[MAXD], orient_f, sarea_f;   // FP32 roundings
    float pad_f;            // zero (keeps the record free of implicit padding)
    // a face to a SolidNeighbor record: the reconstruction perturbance's lever arm
    // x_solid[dir] - x_aux[dir] (update_solid_neighbor!, Immersed_boundary.jl:477), which
    // positivity_preserving_ib! reads under CIP marching
    double pert;
    float pert_f;
    int32_t wallrec;        // 1 for such a face
};

// What the flux kernel needs of a fluid cell before its first barrier, in one record
// (built when the problems are merged).
struct FluxCell {
    int64_t foff;           // f offset of the cell
    int64_t goff;           // first velocity cell of its grid
    double invV;            // 1 / cell volume
    double ds[MAXD];
    int32_t cell, slot, inc0, ninc;
    int32_t nv, gid, reg, pad;
};

// The faces of a regular fluid cell (fluid_reg), by side s = 2 * dir + (face at +ds/2): the
// neighbour across it (f offset; its sdf is at nfo * dim), the face midpoint minus the cell
// centre along dir, and the signed area factor of the received flux, in FP64 and rounded to
// FP32 (built when the problems are merged; zero for cells that are not regular).
struct RegRec {
    int64_t nfo[2 * MAXD];
    double dxm[2 * MAXD], sa[2 * MAXD];
    float dxm_f[2 * MAXD], sa_f[2 * MAXD];
    int32_t nd[2 * MAXD];   // the neighbours' data indices
};

// A regular 2D cell whose four neighbours are regular too, in the slope sense as well: the
// flux kernel computes its own slopes and its neighbours' from f (the regular slope formula,
// the same bits as slope_kernel), so neither reads nor needs sdf.  Per side s of the cell
// (2 * dir + (face at +ds/2)): that neighbour's own four neighbours (f offsets, by its sides)
// and its slope factors; the cell's own slope factors.
struct R2Rec {
    int64_t nn[4][4];
    float ninv[4][4];
    float sinv[4];
};

// ---- immersed boundary ----------------------------------------------------
struct SolidOp {            // update_solid_cell! for one solid cell
    int32_t cell, list, cnt, pad;
};
struct WallOp {             // update_solid_neighbor! for one SolidNeighbor
    double ib_point[MAXD], aux[MAXD], normal[MAXD], bc[MAXW];
    double dxf, dxs, dxL;
    int32_t donor, solid, data, dir;
    int32_t list, cnt;      // image_df sources (fluid neighbours + donor) in ib_nbr
    int32_t spair;          // pairing (donor grid <- solid grid) for boundary_slope!
    int32_t cut_off, cut_cnt;
    int64_t cvcw_off;       // dense cut-cell weight vector (weight with cut cells zeroed)
};

// ---- per-problem parameters (a handle advances one or many independent problems) --
struct ProbParams {
    double gamma, K, Pr, omega, mu_ref, dt;
    int32_t check;                 // st_check_interval
    int32_t fluid_begin, fluid_end; // range of the problem in the merged fluid-cell list
    int32_t slot;
    // FP32 copies for the mixed form's per-cell constants: dt, K, 2 mu_ref, 1 - omega, 0.8 (1 - Pr)
    float dtf, Kf, mu2f, omf, shkf;
};

// ---- flattened topology (host copy, then mirrored to device) ------------------
struct Flat {
    int dim = 2, ndf = 2;
    int n_cells = 0, n_walls = 0, n_data = 0;
    int n_fluid = 0;              // cells with bound_enc >= 0
    int64_t phase_cells = 0;      // Σ nv over fluid cells
    int max_nv = 0;
    // velocity grids
    std::vector<int64_t> g_off;   // n_grids + 1
    std::vector<int8_t> vlev;
    std::vector<double> vw;
    std::vector<double> vu;       // [dim][P_g] (dimension-major)
    std::vector<float> vuf, vwf;  // FP32 copies for the mixed form
    // factorised Maxwellian: per grid and dimension the distinct midpoint coordinates
    // ("axis values") and, per velocity cell, the index of its coordinate on each axis
    std::vector<int32_t> ax_off;  // n_grids * MAXD + 1
    std::vector<double> ax_val;
    std::vector<float> ax_hi, ax_lo;   // ax_val = hi + lo in FP32 pairs (mixed form exponents)
    std::vector<uint16_t> vidx;   // [dim][P_g]
    int max_axis = 0;
    // data table
    std::vector<int64_t> foff;    // n_data + 1, element offsets (ndf * nv blocks)
    std::vector<int32_t> dgrid, dbe;
    std::vector<double> dinvv;    // n_data: 1 / cell volume (Π ds)
    std::vector<int32_t> dnv;      // velocity cells per data item
    std::vector<int32_t> dprob;    // problem slot per data item
    std::vector<double> dmid, dds; // n_data * MAXD
    // pairing tables
    std::vector<int64_t> p_off;    // n_pairs + 1 (offsets into p_j0 / p_cnt)
    std::vector<int32_t> p_j0, p_cnt;
    // slope: passes (by dependency depth: the first holds every cell that reads f alone) and ops
    std::vector<int32_t> pass_off;   // per level + 1 into slope_ops (the ops' build order)
    std::vector<SlopeOp> slope_ops;  // ordered by level, then cell, then dir
    std::vector<int32_t> pass_cells_off;  // per pass: cells [pass_cells_off[p], ...) in pass_cells
    std::vector<int32_t> pass_cells;
    std::vector<int32_t> cell_slope_op;   // per pass-cell entry: first op index (dim ops each)
    std::vector<int32_t> slope_items;     // merged layout: (pass-cell entry, velocity chunk) pairs
    std::vector<int32_t> pass_items_off;  // merged layout: per pass its items (one CTA each), then
                                          // one entry more: the end of the lazy items (the slopes a
                                          // step does not need, computed only at sync points)
    std::vector<NbrRef> slope_nbr;
    // flux incidences, per fluid cell
    std::vector<int32_t> fluid_cells;     // fluid cell ids (bound_enc >= 0), flux/collide order
    std::vector<FluxCell> fcrec;          // merged layout only: per fluid cell
    std::vector<RegRec> regrec;           // merged layout only: per fluid cell (regular ones filled)
    std::vector<uint8_t> fluid_r2;        // merged layout only: per fluid cell, 1 = slopes computed in
                                          // the flux kernel (R2Rec), 2 = besides, no other cell reads its
                                          // slopes in a step (they leave the slope passes: lazy items)
    std::vector<R2Rec> r2rec;             // merged layout only: per fluid cell (fluid_r2 > 0 filled)
    std::vector<SlopeCell> screc;         // merged layout only: per pass-cell entry
    std::vector<CritOp> crit_ops;         // per fluid cell and direction (fluid-list order)
    std::vector<int32_t> crit_nbr;        // their neighbour lists (data indices)
    std::vector<uint8_t> fluid_reg;       // per fluid cell: 1 when its faces are 2*dim full inner faces
                                          // to same-sized neighbours on the same velocity grid
    std::vector<int32_t> inc_off;         // n_fluid + 1
    std::vector<Incidence> inc;
    std::vector<double> bc_prim;          // domain-face bc prim, MAXW per entry
    std::vector<float> bc_hl;             // the same as FP32 hi (MAXW) then lo (MAXW) per entry
    // immersed boundary
    std::vector<SolidOp> solid_ops;
    std::vector<WallOp> wall_ops;
    std::vector<NbrRef> ib_nbr;
    std::vector<double> ib_dx;            // per ib_nbr entry: dx[MAXD] (target - source centre)
    std::vector<int32_t> cut_idx;
    std::vector<double> cut_gw, cut_sw;
    std::vector<double> cvcw;
    int max_inc = 0;
    int max_bcm = 0;                      // most Maxwellian-state domain faces (wall, inflow) of a cell
    // the arrays a step reads beyond these (slope ops and lists, criterion rows, incidences,
    // per-cell records) were built on the device (kg_devflat.cu) and live there only
    bool devlay = false;
};

// One cell of an adapted mesh and the cells of the previous mesh its state comes from
// (ps_replace!, Physical_space/AMR.jl:633-703), resolved to pool positions on the host.
// kind: KG_ADAPT_KEEP (src 0), KG_ADAPT_REFINE (src 0 = the parent, `depth` refinements
// along `path`), KG_ADAPT_COARSEN (srcs 0..2^dim-1 = the children in RMT order).
struct AdaptRec {
    int64_t src_f[8];      // f element offset of each source block in the previous pools
    int64_t run[8];        // COARSEN: first (j0, count) pair of the child's runs; -1: same grid
    int64_t lev[8];        // COARSEN: offset of the child's grid levels in the level table
    double ds[MAXD];       // REFINE: the parent's ds
    int32_t src_nv[8];     // velocity cells of each source
    int32_t src_d[8];      // data index of each source in the previous pools (w, prim, qf rows)
    int32_t cell;          // data index of the new cell (merged layout)
    int32_t kind, depth, nsrc;
    int8_t path[8];        // REFINE: child number (RMT order, bit d = upper half in dim d)
};

// Arguments of the velocity-space flag kernel (see kg_vs_flags).
struct VsFlagArgs {
    const int32_t* nbr;      // per velocity cell of every grid: 2*dim face neighbours (grid-local, -1: none)
    uint8_t* flags;          // per velocity cell of the problem's cells, in cell order
    double* eta;             // the same rows, or null
    int64_t row0;            // f offset of the problem's first cell (rows = f offset / ndf)
    double hf[MAXD];         // finest velocity-cell size per dimension
    double dens_res, en_res; // Velocity_Resolution
    double tau_l, tau_c, c_local, c_global;
    int maxlevel, lohner;
};

// Same-or-coarser face neighbours in velocity space (vs_face_neighbor,
// Velocity_space/Neighbor.jl:181-204) of every velocity cell of the layout's grids: 2*dim
// grid-local leaf indices per cell (-1 across the velocity-domain edge).
void vs_face_table(const Flat& M, const double* vmin, const double* hf, const int32_t* trees, int maxlevel,
                   std::vector<int32_t>& nbr);

// The level merge walk of two velocity grids (diff_vs!, vs_merge!): per cell of grid A the
// (first, count) run of grid-B cells overlapping it.  False when the grids do not tile the
// same root lattice.
bool level_runs(const int8_t* la, int na, const int8_t* lb, int nb, int D, std::vector<int32_t>& runs);

// Empties a gather form, keeping the capacity of its arrays for the next build.
void reset(Flat& F);

// The canonical velocity pairings of one topology (build_pairs): every (my grid, its grid)
// pair that a neighbour reference, an inner face or a wall record relates, numbered by
// ascending (my grid, its grid); and the coarsest and finest fluid-cell levels.
struct PairIds {
    int G = 0;
    std::vector<int32_t> dense;              // G x G ids (-1: none) when G <= 1024
    std::map<std::pair<int, int>, int> ids;  // otherwise
    int lmin = 0, lmax = 0;
    void clear() { G = 0; dense.clear(); ids.clear(); lmin = lmax = 0; }
    int find(int ga, int gb) const;
};
int build_pairs(const kg_topology& t, Flat& F, PairIds& pid, std::string& err);

// The part of the gather form both builders share: argument and topology checks, the velocity
// grids and their axis tables, the data table, the fluid-cell count and levels, and the
// pairing tables (F.p_*).
int flatten_head(const kg_params& prm, const kg_topology& t, Flat& F, PairIds& pid, std::string& err);
// The face-list checks the host builder makes while placing incidences (same order, messages).
int flatten_checks(const kg_params& prm, const kg_topology& t, const Flat& F, std::string& err);
// The immersed-boundary records (solid_ops, wall_ops, ib_nbr, ib_dx, cut_*, cvcw).
int flatten_ib(const kg_topology& t, Flat& F, const PairIds& pid, std::string& err);

// Builds the gather form; returns KG_OK or an error code with a message.
int flatten(const kg_params& prm, const kg_topology& t, Flat& out, std::string& err);

// One problem of a batch: its own flattened topology placed at data slots
// [dbase, dbase + n_data) and f elements [fbase, fbase + foff.back()) of the pools.
struct Part {
    const Flat* F;
    int64_t fbase;
    int32_t dbase;
    int32_t slot;
};
// Concatenates the parts into one gather form whose data indices are pool positions
// (dcap slots); fills the fluid range of every part into `ranges` (begin, end pairs).
// fuse: 2D layouts of the packed regular-cell kernel, which computes the slopes of its R2 cells
// light: the parts' step arrays were built on the device (Flat::devlay); only the host-side
// arrays are merged, and the slope work items are left to slope_items()
void merge(const std::vector<Part>& parts, int32_t dcap, Flat& out, std::vector<int32_t>& ranges, bool fuse,
           bool light = false);
// The work items of the slope passes of a merged layout, from its pass cells and fluid_r2.
void slope_items(Flat& M, int32_t dcap, bool fuse);
int64_t device_bytes(const Flat& f, int precision);

}  // namespace kg
