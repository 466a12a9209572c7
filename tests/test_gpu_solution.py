"""save_result's rows from the device state (kg_download_solution) against the oracle's
restatement of save_result (IO/Output.jl:198-255): PS_Solution prim / qf per quadrant in the
reference's quadrant order (NaN rows for solid cells and InsideSolidData quadrants) and the
Boundary_PS_Solution of every SolidNeighbor (Boundary/Immersed_boundary.jl:12-61: prim, qf
and the pressure tensor of the wall distribution rebuilt at the aux point).  The output
changes the state as save_result does (fresh slopes, updated solid cells, refreshed
wall-direction slopes), so a step after it is compared too."""
import numpy as np
import pytest

from kitgpu import abi, cases
from parity import ORACLE_THREADS, TOL_FP64, TOL_MIXED, f_error, moment_errors

pytestmark = pytest.mark.gpu

CASES = [
    ("cylinder_ib_adapted", lambda: cases.cylinder(scale=0.25, nv=24, vs_levels=2), 3),
    ("sphere3d_ib", lambda: cases.sphere(scale=0.25, nv=8), 2),
]


def _col_err(got, exp):
    """Largest error of each column relative to that column's largest magnitude."""
    scale = np.maximum(np.max(np.abs(exp), axis=0), 1e-300)
    return float(np.max(np.max(np.abs(got - exp), axis=0) / scale))


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED])
@pytest.mark.parametrize("name,make,nsteps", CASES, ids=[c[0] for c in CASES])
def test_solution_rows_match_oracle(name, make, nsteps, prec):
    import oracle as O
    from kitgpu.solver import GpuStep
    p = make()
    topo, state = cases.build(p)
    dt = p.dt()
    prm64 = abi.make_params(p, precision=abi.KG_PREC_FP64, st_check_interval=1)
    ref = O.OracleState(topo, state).run(prm64, dt, 0, nsteps, nthreads=ORACLE_THREADS)
    g = GpuStep(abi.make_params(p, precision=prec, st_check_interval=1), topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    g.step(dt, 0, nsteps)
    qi, nq = topo["cell_quad"], int(topo["n_quads"])
    got = g.download_solution(quad_index=qi, n_quads=nq)
    exp = ref.solution(prm64, quad_index=qi, n_quads=nq, nthreads=ORACLE_THREADS)
    assert topo["n_walls"] > 0 and nq > topo["n_cells"], "the case has walls and inside-solid quadrants"
    for key in ("prim", "qf"):
        assert np.array_equal(np.isnan(got[key]), np.isnan(exp[key])), key
    tol = 1e-11 if prec == abi.KG_PREC_FP64 else TOL_MIXED
    ok = ~np.isnan(exp["prim"][:, 0])
    assert _col_err(got["prim"][ok], exp["prim"][ok]) <= tol
    assert _col_err(got["walls"], exp["walls"]) <= tol, (name, got["walls"][:2], exp["walls"][:2])
    # the state after the output steps on as the reference's does
    g.step(dt, nsteps, 1)
    ref.run(prm64, dt, nsteps, 1, nthreads=ORACLE_THREADS)
    out = g.download_state()
    g.close()
    errs = moment_errors(topo, ref.w, ref.prim, ref.qf, out["w"], out["prim"], out["qf"])
    if prec == abi.KG_PREC_FP64:
        errs["f"] = f_error(topo, ref.f, out["f"])
        assert all(v <= TOL_FP64 for v in errs.values()), errs
    else:
        keep = {k: v for k, v in errs.items() if k in ("rho", "T") or k[0] in "Uq"}
        assert all(v <= TOL_MIXED for v in keep.values()), keep
