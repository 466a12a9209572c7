/*
 * kitgpu.h -- C-ABI of libkitgpu.so, the GB300 (sm_103a) implementation of
 * KitAMR.jl's per-step phase-space hot path:
 *
 *     slope!  ->  flux!  (domain faces, inner/hanging faces, immersed-boundary wall)
 *             ->  iterate!  (CAIDVM_Marching / Euler: Shakhov g+ and implicit relaxation)
 *
 * The p4est forest, the AMR criteria, the IB geometry and all I/O stay with the
 * caller.  After every adaptation the caller flattens its cell / neighbour / face
 * objects into a kg_topology (plain arrays, described below) and uploads it; the
 * library owns every device allocation.  All entry points return an int status
 * (KG_OK == 0); nothing throws across the ABI.  One host thread per handle.
 *
 * Reference interfaces replaced (paths relative to the KitAMR.jl project):
 *   slope!(p4est,ka)              src/Flux/Slope.jl:1047-1070
 *   flux!(p4est,ka)               src/Flux/Flux.jl:458-488
 *   iterate!(p4est,ka)            src/Theory/Iterate.jl:5-16 (the per-cell marching
 *                                 kernels at :96-130 and :131-162)
 *   calc_flux / calc_domain_flux  src/Flux/CAIDVM.jl:4-121, src/Flux/DVM.jl:1-99
 *   update_solid_cell!            src/Boundary/Immersed_boundary.jl:122-146,207-213
 *   update_solid_neighbor!        src/Boundary/Immersed_boundary.jl:436-500
 *   residual_check!               src/Solver/Finalize.jl:5-11
 */
#ifndef KITGPU_H
#define KITGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define KG_OK               0
#define KG_ERR_ARG          1   /* bad argument / null pointer / size mismatch      */
#define KG_ERR_TOPOLOGY     2   /* topology rejected (inconsistent or unsupported)  */
#define KG_ERR_CUDA         3   /* CUDA runtime error                                */
#define KG_ERR_NOMEM        4   /* device or host allocation failed                  */
#define KG_ERR_NONFINITE    5   /* device status word: non-finite moment             */
#define KG_ERR_NEGATIVE     6   /* device status word: rho <= 0 or lambda <= 0       */
#define KG_ERR_STATE        7   /* call out of order (e.g. step before upload)      */
#define KG_ERR_BUDGET       8   /* admission refused: HBM footprint over budget      */
#define KG_ERR_TIMEOUT      9   /* bounded device wait gave up                       */

/* ---- scheme selectors (src/Abstract/Types.jl:320-337) -------------------- */
#define KG_FLUX_CAIDVM      0   /* CAIDVM: micro + macro flux, conserved w           */
#define KG_FLUX_DVM         1   /* DVM: micro flux only                              */
#define KG_MARCH_CAIDVM     0   /* iterate!(::Type{CAIDVM_Marching})  Iterate.jl:96  */
#define KG_MARCH_EULER      1   /* iterate!(::Type{Euler})            Iterate.jl:131 */
#define KG_MARCH_CIP        2   /* iterate!(::Type{CIP_Marching}) I-projection.jl:161:
                                   convection, then the conservative I-projection of f
                                   onto w (a Newton solve per cell) before relaxation;
                                   next to immersed-boundary walls with
                                   positivity_preserving_ib! (Boundary/Positivity.jl)  */
#define KG_PREC_FP64        0   /* f, sdf, fluxes in FP64 (plain form)               */
#define KG_PREC_MIXED       1   /* f, sdf, micro fluxes in FP32; moments compensated;
                                   w, prim, exponents, wall density in FP64          */

/* ---- face / boundary kinds --------------------------------------------- */
#define KG_FACE_INNER       0   /* FullFace, or one sub-face of a (Back)HangingFace  */
#define KG_FACE_DOMAIN      1   /* DomainFace                                        */
#define KG_BC_MAXWELL       0   /* Domain(Maxwellian,...)       CAIDVM.jl:4-25       */
#define KG_BC_INFLOW        1   /* Domain(SuperSonicInflow,...) CAIDVM.jl:29-49      */
#define KG_BC_OUTFLOW       2   /* Domain(UniformOutflow,...)   CAIDVM.jl:53-67      */
#define KG_BC_INTERP        3   /* Domain(InterpolatedOutflow)  CAIDVM.jl:71-94 (2D) */

/* neighbour reference encoding inside kg_topology.nbr_ref / face_there */
#define KG_NBR_NONE   INT32_MIN /* `nothing` (domain boundary, state 0)             */
#define KG_NBR_INSIDE (INT32_MIN + 1) /* InsideSolidData (no distribution function) */
#define KG_WALL(w)    (-1 - (w))/* SolidNeighbor record w                            */

/* ---- solver parameters (Gas, Solver, Status of src/Solver/Types.jl) ------ */
typedef struct kg_params {
    int32_t dim;                 /* 2 or 3                                          */
    int32_t ndf;                 /* 2 in 2D (h, b); 1 in 3D                          */
    int32_t flux;                /* KG_FLUX_*                                        */
    int32_t marching;            /* KG_MARCH_*                                       */
    int32_t precision;           /* KG_PREC_*                                        */
    int32_t st_check_interval;   /* solver.ST_CHECK_INTERVAL (residual cadence)      */
    double  gamma;               /* gas.γ                                            */
    double  K;                   /* gas.K  (internal DOF)                            */
    double  Pr;                  /* gas.Pr                                           */
    double  omega;               /* gas.ω  (get_τ exponent, src/Gas/Model.jl:14)     */
    double  mu_ref;              /* gas.μᵣ (as the caller computed it)               */
} kg_params;

/* ---- flattened topology (reference-shaped arrays) ------------------------ *
 * Arrays are read during kg_upload_topology only and never retained.
 *
 * Velocity grids.  Grid g owns velocity cells [grid_off[g], grid_off[g+1]) in the
 * reference's depth-first leaf order (src/Velocity_space/Rebuild.jl:44-85).
 * vs_midpoint for grid g is the column-major nv x dim block starting at
 * grid_off[g]*dim (u of every cell, then v, then w) -- the memory of VsData.midpoint.
 *
 * Cells.  Every PsData that carries a distribution function: fluid cells
 * (bound_enc == 0), IB donor cells (bound_enc > 0) and solid ghost cells
 * (bound_enc < 0).  InsideSolidData carries none and is not listed.
 *
 * Neighbour lists.  For cell c and faceid k (0-based, 2*dim per cell, reference
 * faceid k+1): state nbr_state[c*2*dim+k] in {0, 1, 2^(dim-1), -1}
 * (src/Physical_space/Types.jl:6-9) and references
 * nbr_ref[nbr_off[c*2*dim+k] .. nbr_off[c*2*dim+k+1]) in p4est order; a
 * reference is a cell index, KG_WALL(w) for a SolidNeighbor, KG_NBR_INSIDE for
 * an InsideSolidData, or KG_NBR_NONE.
 *
 * Faces.  The reference face list with every HangingFace / BackHangingFace
 * expanded into its sub-faces (src/Flux/Flux.jl:37-59).  face_area is the signed
 * value update_flux!/update_domain_flux! multiply by (rot * face_area / 2^(dim-1)
 * for a HangingFace sub-face; Flux.jl:64-111).  face_there_midpoint is the
 * midpoint of the across-face data as the face sees it (the shifted copy for a
 * periodic face, Boundary/Period.jl / Solver/Initialize.jl:77-79).
 */
typedef struct kg_topology {
    int32_t dim, ndf;
    /* velocity grids */
    int32_t        n_grids;
    const int64_t *grid_off;         /* n_grids + 1                                  */
    const int8_t  *vs_level;         /* grid_off[n_grids]                            */
    const double  *vs_weight;        /* grid_off[n_grids]                            */
    const double  *vs_midpoint;      /* grid_off[n_grids] * dim (per-grid col-major) */
    /* cells */
    int32_t        n_cells;
    const int32_t *cell_bound_enc;   /* n_cells                                      */
    const int32_t *cell_level;       /* n_cells: physical level (Slope.jl:825-829)   */
    const int32_t *cell_grid;        /* n_cells: velocity grid id                    */
    const double  *cell_midpoint;    /* n_cells * dim (row-major)                    */
    const double  *cell_ds;          /* n_cells * dim                                */
    /* neighbours */
    const int8_t  *nbr_state;        /* n_cells * 2*dim                              */
    const int32_t *nbr_off;          /* n_cells * 2*dim + 1                          */
    const int32_t *nbr_ref;          /* nbr_off[n_cells*2*dim]                       */
    /* immersed-boundary wall records (SolidNeighbor, Physical_space/Types.jl:28-48) */
    int32_t        n_walls;
    const int32_t *wall_donor;       /* donor cell (bound_enc > 0)                   */
    const int32_t *wall_solid;       /* solid ghost cell                             */
    const int32_t *wall_faceid;      /* 0-based faceid of the donor                  */
    const double  *wall_aux_point;   /* n_walls * dim                                */
    const double  *wall_normal;      /* n_walls * dim                                */
    const double  *wall_bc;          /* n_walls * (dim+2): ib.bc at the aux point    */
    const int32_t *wall_cut_off;     /* n_walls + 1: cut velocity cells (CuttedVelocityCells) */
    const int32_t *wall_cut_index;   /* 0-based velocity index in the donor grid     */
    const double  *wall_cut_gas_w;   /* gas_weights                                  */
    const double  *wall_cut_solid_w; /* solid_weights                                */
    /* faces */
    int32_t        n_faces;
    const int8_t  *face_kind;        /* KG_FACE_*                                    */
    const int8_t  *face_dir;         /* 0-based normal direction                     */
    const double  *face_rot;         /* +1 / -1                                      */
    const double  *face_area;        /* signed area factor (see above)               */
    const double  *face_midpoint;    /* n_faces * dim                                */
    const int32_t *face_here;        /* cell index (always a local PsData)           */
    const int32_t *face_there;       /* cell index or KG_WALL(w); unused for domain  */
    const double  *face_there_midpoint; /* n_faces * dim; unused for domain          */
    const int8_t  *face_bc_kind;     /* KG_BC_* for domain faces                     */
    const double  *face_bc;          /* n_faces * (dim+2): bc prim for domain faces  */
} kg_topology;

/* Residual sums of residual_check! (Finalize.jl:5-11) for the last step of the
 * call whose step counter was a multiple of st_check_interval.               */
typedef struct kg_step_report {
    int32_t status;              /* device status word mapped to KG_ERR_*        */
    int32_t checked;             /* 1 if some step of the call was a check step  */
    int64_t checked_step;        /* the step counter of that step                */
    double  sum_res[5];          /* Σ (prim_c - prim_old)^2      (dim+2 used)   */
    double  sum_avg[5];          /* Σ |prim_c|                                    */
    double  device_ms;           /* device time of the whole call (CUDA events)  */
    int64_t phase_cells;         /* Σ velocity cells over fluid + donor cells    */
    int32_t kernel_launches;     /* kernels this call launched                   */
} kg_step_report;

typedef struct kg_handle kg_handle;

/* Lifecycle.  kg_create selects device `device` (-1: current). */
int kg_create(const kg_params *params, int device, kg_handle **out);
int kg_destroy(kg_handle *h);

/* Replaces the topology (after initialize / amr_recover!, Solver/AMR.jl:54-70).
 * Device state is re-allocated and must be uploaded again.                  */
int kg_upload_topology(kg_handle *h, const kg_topology *topo);

/* State transfer.  f: concatenation over cells (in cell order) of the column-
 * major nv x ndf block (VsData.df memory); w, prim: n_cells x (dim+2) row-major.
 * kg_download_state: any output pointer may be NULL; qf is n_cells x dim; sdf is
 * per cell the column-major nv x ndf x dim block (VsData.sdf memory).        */
int kg_upload_state(kg_handle *h, const double *f, const double *w, const double *prim);
int kg_download_state(kg_handle *h, double *f, double *w, double *prim, double *qf, double *sdf);

/* Macroscopic slopes sw of update_macro_slope! (Flux/Slope.jl:1022-1036, the last call of
 * slope!, Slope.jl:1064): for every cell with bound_enc >= 0 and each direction dir,
 * sw[:, dir] = calc_w0 of sdf[:, :, dir].  Computed on demand from the slopes on the device,
 * which are those the last kg_step used, so AMR criteria and output at a sync point read the
 * values PsData.sw holds.  sw: n_cells blocks of (dim+2) x dim doubles, column-major (the
 * PsData.sw memory); solid cells (bound_enc < 0) get zeros.                    */
int kg_download_sw(kg_handle *h, double *sw);

/* Physical-space refinement sensor of the adaptation step: PsData.lohner as
 * update_criterion! leaves it (Physical_space/AMR.jl:256-284; update_Lohner_inner_ps!,
 * Physical_space/Criteria.jl:95-158), including apply_amr_buffer!'s one-cell buffer layer
 * (AMR.jl:286-330) with threshold adapt_coeffi_ps (solver.ADAPT_COEFFI_PS).  As
 * ps_adaptive_mesh_refinement! does (Physical_space/AMR.jl:1108-1116), the slopes are first
 * recomputed from the current f (slope!), then sw and the sensor follow in FP64 from w, prim
 * and that sw; the refreshed slopes stay on the device (kg_download_state's sdf, kg_download_sw,
 * kg_adapt's refinement).  The host applies ps_refine_flag / ps_coarsen_flag (user-defined
 * functions) to the sensor, so only
 * (dim+2) x dim doubles per cell cross the link at an adaptation instead of f.
 * lohner: n_cells blocks of (dim+2) x dim doubles, column-major (PsData.lohner memory);
 * solid cells get zeros.  A direction whose two sides are both coarser uses 1.5 ds on
 * both sides (the reference has no applicable method for that case).          */
int kg_criterion(kg_handle *h, double adapt_coeffi_ps, double *lohner);

/* ---- physical-space adaptation on the device --------------------------------
 * The state moves of the refine / coarsen / balance callbacks (ps_replace!,
 * Physical_space/AMR.jl:633-703), applied to the device state without sending f to the
 * host.  The caller records, in its replacement callbacks, where every cell of the
 * adapted mesh comes from and passes one kg_adapt_src per cell of the new topology (same
 * order as topo's cells):
 *   KG_ADAPT_KEEP     src[0]: the same cell in the previous topology (also the children a
 *                     balance pass restores after a coarsening, BALANCE_FLAG);
 *   KG_ADAPT_REFINE   src[0]: the parent; `depth` refinements (1..KG_ADAPT_MAX_DEPTH, more
 *                     than one under recursive refinement) along path[0..depth-1], each a
 *                     0-based child number in RMT order (Abstract/Types.jl:10: bit d set =
 *                     upper half in dimension d).  Per velocity cell and level, with the
 *                     child's ds (half the parent's):
 *                     df += min(|df / (ds . |sdf| + EPS)|, 1) * (sdf . (ds/2 .* RMT[i]))
 *                     with the parent's slopes; sdf is the parent's; w = calc_w0,
 *                     prim = get_prim; qf = 0;
 *   KG_ADAPT_COARSEN  src[0..2^dim-1]: the children in RMT order.  The parent's velocity
 *                     grid must be the grid of the first child with the fewest velocity
 *                     cells (ps_merge); df and sdf are the vs_merge! sums of the children
 *                     over 2^dim, w the children's mean, prim = get_prim(w), qf = 0;
 *   KG_ADAPT_VS       src[0]: the same cell before a velocity-space adaptation
 *                     (vs_refine! / vs_coarsen!, Velocity_space/AMR.jl:26-118) that gave
 *                     it a new velocity grid, or the same one: refine_grid_stream! and
 *                     coarsen_grid_stream! (Rebuild.jl:44-163) move df -- a refined
 *                     velocity cell's children take its df, 2^dim coarsened siblings their
 *                     mean -- along the level merge walk of the two grids; sdf is zero (both
 *                     streams reset it), w, prim and qf are kept.  The conservative
 *                     correction that follows is kg_vs_conserve.
 * Indices refer to the cells of the topology on the device before the call; KEEP and
 * REFINE cells keep their source's velocity grid (equal content).  As
 * ps_adaptive_mesh_refinement! does, the slopes of the current f are recomputed first
 * (slope!).  After the call the handle holds the new topology and state (walls start
 * from their donors' f, as after amr_recover!), exactly as kg_upload_topology +
 * kg_upload_state with the interpolated state would leave it.  Device memory peaks at
 * the previous plus the new pools during the call.  A rejected plan (KG_ERR_ARG: a source
 * out of range, a bad depth or child number; KG_ERR_TOPOLOGY: a grid that breaks the rules
 * above, or a new topology flatten rejects) leaves the handle as it was; a device failure
 * after that (KG_ERR_NOMEM, KG_ERR_CUDA) leaves it without a state.                   */
#define KG_ADAPT_KEEP       0
#define KG_ADAPT_REFINE     1
#define KG_ADAPT_COARSEN    2
#define KG_ADAPT_VS         3
#define KG_ADAPT_MAX_DEPTH  8
typedef struct {
    int32_t kind;
    int32_t depth;
    int32_t src[8];
    int8_t  path[KG_ADAPT_MAX_DEPTH];
} kg_adapt_src;
int kg_adapt(kg_handle *h, const kg_topology *topo, const kg_adapt_src *src);

/* ---- velocity-space adaptation flags on the device ---------------------------------------
 * The per-velocity-cell decisions of vs_refine! / vs_coarsen! (Velocity_space/AMR.jl:26-118)
 * computed from the device state, so the host's loops over every phase cell become one
 * download of Nv bytes:
 *   bit 0  refine:     level < maxlevel and, in KG_VS_LOHNER mode, the Löhner indicator
 *                      (vs_lohner_indicator, Velocity_space/Criteria.jl:253-283) above
 *                      coeffi_lohner or local_contribution_refine_flag; in KG_VS_CONTRIBUTION
 *                      mode contribution_refine_flag (local or global, Criteria.jl:4-58);
 *   bit 1  coarsen_ok: the indicator below 0.3 coeffi_lohner (VS_LOHNER_COARSEN_RATIO) and
 *                      local_contribution_coarsen_flag (Löhner mode), or the local and global
 *                      coarsen flags (contribution mode), for the cell's single velocity cell.
 * The contribution flags read the criterion distribution df + max_d |sdf ds_d| of
 * _criterion_cell! (the slopes on the device, as the reference reads PsData's) and, for the
 * global ones, the Velocity_Resolution of vs_resolution (AMR.jl:135-166), returned in vr[2].
 * Both bits are those of the grid on the device: the reference evaluates coarsening after its
 * refinement pass, so bit 1 is final for cells with no bit 0 set.  Every cell with a
 * distribution (solid ghost cells included, as vs_refine! visits them) gets its nv bytes, in
 * cell order (Σ nv bytes); eta (optional) receives the indicator per velocity cell (Löhner
 * mode; zeros otherwise).  Face neighbours in velocity space are the same-or-coarser leaves of
 * vs_face_neighbor (Velocity_space/Neighbor.jl:181-204), the domain edge counting as vacuum.
 * Arithmetic in FP64 from the stored f (FP32 in the mixed form).                         */
#define KG_VS_LOHNER        0   /* ADAPT_VS_MODE = :lohner (the reference's default)     */
#define KG_VS_CONTRIBUTION  1   /* any other mode: the contribution flags                 */
typedef struct {
    double  quadrature[6];     /* config.quadrature: (lower, upper) per dimension            */
    int32_t vs_trees_num[3];
    int32_t maxlevel;          /* solver.AMR_VS_MAXLEVEL                                    */
    int32_t mode;              /* KG_VS_*                                                    */
    int32_t pad;
    double  coeffi_lohner;     /* solver.ADAPT_COEFFI_VS_LOHNER (default 0.6)               */
    double  coeffi_local;      /* solver.ADAPT_COEFFI_VS_LOCAL (default 1e-2)               */
    double  coeffi_global;     /* solver.ADAPT_COEFFI_VS_GLOBAL (default 0.125)             */
} kg_vs_config;
int kg_vs_flags(kg_handle *h, const kg_vs_config *cfg, uint8_t *flags, double *eta, double *vr);

/* vs_conserved_correction! (Velocity_space/AMR.jl:122-137) on the device state: for every cell
 * c with cell_flags[c] != 0 (n_cells bytes; solid cells are skipped), conserved_I_porjection!
 * (Theory/I-projection.jl:144-158) of its f onto its w -- the Newton solve of
 * solve_I_projection (:55-141) with the negative-value shave, then f₁ *= exp(λ·ψ).  For a
 * caller that rebuilt velocity grids (vs_refine! / vs_coarsen!) and uploaded the new state, or
 * any state whose moments must be made to match w.                                        */
int kg_vs_conserve(kg_handle *h, const uint8_t *cell_flags);
int kg_batch_vs_conserve(kg_handle *h, int32_t slot, const uint8_t *cell_flags);   /* kg_vs_conserve of one problem */
int kg_batch_vs_flags(kg_handle *h, int32_t slot, const kg_vs_config *cfg, uint8_t *flags, double *eta,
                      double *vr);   /* kg_vs_flags of one problem (vr over that problem) */

/* ---- checkpoint payload from the device (save_for_restart / restart, IO/Restart.jl) --------
 * kg_download_restart fills the per-rank arrays of restart_<rank>.jld2 that come from the
 * state (IO/Restart.jl:81-117), in FP64:
 *   vs_df  the Nv x ndf column-major matrix of every cell's VsData.df stacked in cell order
 *          (Nv = the sum of the cells' velocity-cell counts; column k holds df[:, k]);
 *   ws     the n_quads x (dim+2) column-major matrix of PsData.w, row quad_index[c] for cell
 *          c; rows of quadrants without a distribution function (InsideSolidData) are zero.
 * quad_index may be NULL (row c for cell c; n_quads must then equal n_cells); either output
 * may be NULL.  vs_nums, bound_encs, vs_levels and vs_midpoints are topology the caller holds.
 * kg_upload_restart is the inverse as restart() builds its PsData (IO/Restart.jl:300-325):
 * f from vs_df, w from ws, prim = get_prim(w) (on the device), qf and slopes zero, walls from
 * their donors; the topology must be uploaded first.  Together they resume a run bit for bit
 * in the FP64 form (the mixed form stores f in FP32).                                     */
int kg_download_restart(kg_handle *h, const int32_t *quad_index, int32_t n_quads, double *vs_df, double *ws);
int kg_upload_restart(kg_handle *h, const int32_t *quad_index, int32_t n_quads, const double *vs_df,
                      const double *ws);

/* ---- save_result rows from the device state (IO/Output.jl:198-255) ----------------------
 * As save_result first runs update_slope! and update_solid_cell!, the slopes are recomputed
 * from the current f and the solid cells updated (state changes the reference makes too).
 *   ps_prim   n_quads x (dim+2) row-major: PS_Solution.prim (IO/Types.jl:56-68) of every
 *             quadrant, row quad_index[c] for cell c; NaN for cells with bound_enc < 0 and for
 *             quadrants without a cell (InsideSolidData)
 *   ps_qf     n_quads x dim, the same for PS_Solution.qf
 *   wall_rows per SolidNeighbor record (topology order) its Boundary_PS_Solution of
 *             save_boundary_result! (Boundary/Immersed_boundary.jl:12-61): prim (dim+2), qf (dim)
 *             and the pressure tensor p (2D: p11 p12 p22; 3D: p11 p12 p13 p22 p23 p33) of the
 *             wall distribution rebuilt at the aux point -- 9 doubles a row in 2D, 14 in 3D.  As
 *             in the reference the record's wall-direction slope is refreshed and its
 *             distribution left as it was.
 * quad_index may be NULL (n_quads must then equal n_cells); any output may be NULL.  The
 * VS_Solution rows are kg_download_state's f; the JLD2 / VTK writers stay with the caller.   */
int kg_download_solution(kg_handle *h, const int32_t *quad_index, int32_t n_quads, double *ps_prim,
                         double *ps_qf, double *wall_rows);

/* Advance `nsteps` steps with time step dt; `step` is status.step before the
 * first of them (drives the residual cadence).  One call = nsteps x
 * (slope -> flux -> iterate).                                               */
int kg_step(kg_handle *h, double dt, int64_t step, int32_t nsteps, kg_step_report *report);

/* Pipelined serving of independent requests on the uploaded topology (single-problem
 * handle).  Request r starts from the host state f_in[r], w_in[r], prim_in[r] (layouts of
 * kg_upload_state), advances nsteps steps from step counter step0 with time step dt, and
 * writes its final state to f_out[r], w_out[r], prim_out[r], qf_out[r] (layouts of
 * kg_download_state; an output array or entry may be NULL) and its report to reports[r].
 * The result equals kg_upload_state + kg_step + kg_download_state per request, bit for bit;
 * the upload of request r+1 and the download of request r-1 run on two copy streams while
 * request r steps, so with pinned host buffers the link carries both directions at once.
 * Returns when every output is written; the handle then holds the last request's state.
 * No counterpart in the reference (a serving loop over its step).                      */
int kg_serve(kg_handle *h, int32_t n_requests, const double *const *f_in, const double *const *w_in,
             const double *const *prim_in, double dt, int64_t step0, int32_t nsteps,
             double *const *f_out, double *const *w_out, double *const *prim_out, double *const *qf_out,
             kg_step_report *reports);

/* Optional per-kernel device timing (CUDA events on the handle's stream).
 * kg_profile_read fills up to `cap` entries; names are static strings.
 * kg_profile_units: per entry (same order) the phase cells its launches
 * processed, summed over the launches (the flux kernels; 0 for the others). */
int kg_profile_enable(kg_handle *h, int enable);
int kg_profile_read(kg_handle *h, const char **names, double *total_ms, int64_t *launches,
                    int32_t cap, int32_t *count);
int kg_profile_units(kg_handle *h, int64_t *units, int32_t cap, int32_t *count);

/* Device bytes held by the handle, and the bytes a topology would need.     */
int kg_memory_footprint(const kg_handle *h, int64_t *bytes);
int kg_topology_footprint(const kg_params *params, const kg_topology *topo, int64_t *bytes);

/* Last error message of the handle (or of the last failed kg_create if h is NULL). */
int kg_last_error(const kg_handle *h, char *buf, size_t cap);

/* Capture the kg_step sequence of `nsteps` steps as a CUDA graph; kg_step then
 * replays it when called again with the same nsteps on the same layout (dt and
 * the step counter live on the device, so a replay uses their current values). */
int kg_use_graph(kg_handle *h, int enable);

/* Autotuner of the flux+collision schedule (one CTA per cell, or a persistent grid of
 * resident CTAs taking cells from a work queue in cell order or largest-grid-first, at
 * the occupancy limit or one CTA/SM below).  When enabled, the first step after each
 * topology or membership change times the candidates on the live layout and keeps the
 * fastest.  All candidates compute every cell identically, so results do not depend on
 * the choice.  kg_autotune_result: chosen schedule (0/1/2), CTAs/SM, per-candidate ms. */
int kg_autotune(kg_handle *h, int enable);
int kg_autotune_result(const kg_handle *h, int32_t *schedule, int32_t *ctas_per_sm, double *trial_ms, int32_t cap);

/* Slopes in the flux kernel (2D mixed form, CAIDVM or Euler marching; default off).  A regular
 * cell whose four neighbours are regular has its slopes and its upwind neighbours' slopes
 * computed in the flux kernel from f (the slope passes' arithmetic, the same bits), so it reads
 * no sdf; when its neighbours are such cells too, no cell reads its slopes in a step and they
 * leave the slope passes (sdf of such cells is filled in only where a call reads the slopes:
 * kg_download_state's sdf, kg_download_sw, kg_vs_flags, or a call that recomputes them).
 * Off: every slope goes through the slope passes and sdf.  Results do not depend on the
 * setting.  On moves less DRAM traffic per step but, on GB300, takes longer (the flux kernel
 * issues more instructions and waits on longer chains of loads).                        */
int kg_fuse_slopes(kg_handle *h, int enable);

/* Builder of the gather form: after kg_upload_topology, kg_batch_admit and kg_adapt
 * (amr_recover!'s rebuild of faces and neighbours, Solver/AMR.jl:54-70, from
 * initialize_faces!, Solver/Initialize.jl:5-158) the slope operations and their neighbour
 * lists, the slope-pass order, the criterion rows, the face incidences and the per-cell flux
 * and slope records are built on the device (enable = 1, the default) or on the host (0).
 * Both give the same arrays byte for byte (kg_layout_read).  A batch handle merges its
 * problems' device-built arrays on the device; its builder can change only while it holds no
 * problem (KG_ERR_STATE otherwise).                                                     */
int kg_device_flatten(kg_handle *h, int enable);

/* Test support: copies the named array of the gather form the next step reads ("slope_ops",
 * "slope_nbr", "cell_slope_op", "pass_cells", "screc", "crit_ops", "crit_nbr", "inc_off",
 * "inc", "bc_prim", "bc_hl", "fluid_cells", "fluid_reg", "fcrec", "regrec", "r2rec",
 * "slope_items", "reg_list", "nonreg_list", "r2_list", "inner_list", "innerp_list", "p_off", "p_j0", "p_cnt", "ib_nbr",
 * "wall_ops", "solid_ops") into out, up to cap bytes; *bytes receives the array's size.
 * No counterpart in the reference (it exposes its Julia objects instead).               */
int kg_layout_read(kg_handle *h, const char *name, void *out, int64_t cap, int64_t *bytes);

/* ---- batches --------------------------------------------------------------
 * Many independent problems (uneven cell and velocity counts, their own gas constants,
 * Δt and step counters) advanced together: every sub-step is one launch over all of
 * them.  A batch handle owns one pool of `pool_bytes` for f / sdf; kg_batch_admit places
 * a problem in a free slot or returns KG_ERR_BUDGET when its footprint does not fit;
 * kg_batch_release frees it.  Problems that stay keep their device state across
 * admissions and releases.  params: dim, ndf, flux, marching, precision are those of
 * every problem of the batch (the gas fields of kg_batch_create's params are unused).
 * reports[slot] receives each live problem's report (cap: length of `reports`).     */
int kg_batch_create(const kg_params *params, int device, int64_t pool_bytes, kg_handle **out);
int kg_batch_admit(kg_handle *h, const kg_params *params, const kg_topology *topo, const double *f,
                   const double *w, const double *prim, double dt, int64_t step, int32_t *slot);
int kg_batch_release(kg_handle *h, int32_t slot);
int kg_batch_step(kg_handle *h, int32_t nsteps, kg_step_report *reports, int32_t cap);
int kg_batch_download(kg_handle *h, int32_t slot, double *f, double *w, double *prim, double *qf);
int kg_batch_download_sw(kg_handle *h, int32_t slot, double *sw);   /* kg_download_sw of one problem */
int kg_batch_criterion(kg_handle *h, int32_t slot, double adapt_coeffi_ps, double *lohner);   /* kg_criterion of one problem */
/* kg_adapt of one problem: its new slabs are placed while the previous ones are live, then
 * the previous ones are released (KG_ERR_BUDGET when the pool cannot hold both).            */
int kg_batch_adapt(kg_handle *h, int32_t slot, const kg_topology *topo, const kg_adapt_src *src);
int kg_batch_download_restart(kg_handle *h, int32_t slot, const int32_t *quad_index, int32_t n_quads,
                              double *vs_df, double *ws);   /* kg_download_restart of one problem */
int kg_batch_info(const kg_handle *h, int32_t *n_live, int64_t *f_free_elems, int64_t *bytes_per_elem);
int kg_batch_set_dt(kg_handle *h, int32_t slot, double dt);

/* Residual sums without any device allocation (no counterpart in the reference).
 * Computes Σ_c (prim_new - prim_old)^2 and Σ_c |prim_new| (the two sums of
 * residual_check!) over n_cells cells of row-major n_cells x (dim+2) device arrays and
 * writes 2*(dim+2) doubles (the squared differences, then the magnitudes) to the device
 * array `sums`, asynchronously on `stream` (NULL: the legacy default stream).
 * For callers that cannot allocate device memory where they need the residual: a host
 * runtime whose device memory belongs to its own pool allocator, or a serving loop that
 * must not let an allocation synchronise the device while other problems run.  Its
 * scratch is a fixed file-scope device array (80 KiB, held by every GPU that loads the
 * library until exit); n_cells above 4,194,304 is rejected with KG_ERR_ARG.  The first
 * call on a device resolves that array's device address (make it before any stream
 * capture) and keeps it for the life of the process: do not cudaDeviceReset a device
 * this is used on.  Calls share the array, so calls that overlap on the GPU race; each call
 * writes every scratch row it reads, so no state carries over between calls.
 * Errors: kg_last_error(NULL, ...).                                           */
int kg_residual_sums_noalloc(const double *prim_new, const double *prim_old, int64_t n_cells,
                             int32_t dim, double *sums, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* KITGPU_H */
