"""GPU parity through the C-ABI: libkitgpu.so against the FP64 oracle on the same inputs."""
import numpy as np
import pytest

from kitgpu import abi, cases
from parity import TOL_FP64, TOL_MIXED, f_error, moment_errors, run_pair

pytestmark = pytest.mark.gpu

CASES_FP64 = [
    ("couette", lambda: cases.couette(n=12, nv=16), 6),
    ("cavity_levels", lambda: cases.cavity(n=8, nv=16, levels=2), 6),
    ("sod_levels", lambda: cases.sod(scale=0.125, nv=16), 6),
    ("cylinder_ib_adapted", lambda: cases.cylinder(scale=0.25, nv=24, vs_levels=2), 4),
    ("box3d_levels", lambda: cases.box3d(n=(6, 4, 4), nv=8, levels=1), 4),
    ("sphere3d_ib", lambda: cases.sphere(scale=0.25, nv=8), 3),
    # 36^2 velocity grids (mean above 1024 velocity cells): the 256-thread flux and slope
    # kernels; the cases above run the 128-thread ones
    ("sod_v36_256_threads", lambda: cases.sod(scale=0.125, nv=36), 4),
]


@pytest.mark.parametrize("name,make,nsteps", CASES_FP64, ids=[c[0] for c in CASES_FP64])
def test_fp64_caidvm_matches_oracle(name, make, nsteps):
    topo, ref, out, rep = run_pair(make(), nsteps)
    errs = moment_errors(topo, ref.w, ref.prim, ref.qf, out["w"], out["prim"], out["qf"])
    errs["f"] = f_error(topo, ref.f, out["f"])
    bad = {k: v for k, v in errs.items() if not v <= TOL_FP64}
    assert not bad, f"{name}: {bad}"
    assert rep.kernel_launches > 0
    # residual sums of the last checked step
    nw = topo["dim"] + 2
    # (a component that is rounding noise everywhere, e.g. (ΔV)^2 ~ 1e-33, gets an absolute floor)
    sr = np.array(rep.sum_res[:nw])
    assert np.allclose(sr, ref.sum_res[:nw], rtol=1e-9, atol=1e-9 * np.max(ref.sum_res[:nw]))
    assert np.allclose(np.array(rep.sum_avg[:nw]), ref.sum_avg[:nw], rtol=1e-11, atol=1e-12 * np.max(ref.sum_avg[:nw]))


@pytest.mark.parametrize("flux,march", [(abi.KG_FLUX_CAIDVM, abi.KG_MARCH_EULER), (abi.KG_FLUX_DVM, abi.KG_MARCH_EULER)])
def test_fp64_euler_and_dvm(flux, march):
    p = cases.sod(scale=0.125, nv=16)
    topo, ref, out, rep = run_pair(p, 4, flux=flux, march=march)
    errs = moment_errors(topo, ref.w, ref.prim, ref.qf, out["w"], out["prim"], out["qf"])
    errs["f"] = f_error(topo, ref.f, out["f"])
    bad = {k: v for k, v in errs.items() if not v <= TOL_FP64}
    assert not bad, bad


def test_fp64_chunked_calls_and_graph_match_single_call():
    p = cases.cylinder(scale=0.25, nv=16, vs_levels=1)
    topo, ref, out1, _ = run_pair(p, 6, chunks=1)
    _, _, out2, _ = run_pair(p, 6, chunks=3)
    _, _, out3, _ = run_pair(p, 6, chunks=3, graph=True)
    assert np.array_equal(out1["f"], out2["f"])
    assert np.array_equal(out1["f"], out3["f"])
    assert f_error(topo, ref.f, out1["f"]) <= TOL_FP64


MIXED = CASES_FP64[:4] + CASES_FP64[5:] + [
    # a 24^3 velocity grid: the mixed flux kernel stages its convected f in the cells' output
    # blocks (shared memory would cost a resident CTA per SM)
    ("sphere3d_v24_global_staging", lambda: cases.sphere(scale=0.25, nv=24), 2),
]


@pytest.mark.parametrize("name,make,nsteps", MIXED, ids=[c[0] for c in MIXED])
def test_mixed_within_1e5_of_fp64(name, make, nsteps):
    topo, ref, out, rep = run_pair(make(), nsteps, precision=abi.KG_PREC_MIXED)
    errs = moment_errors(topo, ref.w, ref.prim, ref.qf, out["w"], out["prim"], out["qf"])
    keep = {k: v for k, v in errs.items() if k in ("rho", "T") or k.startswith("U") or k.startswith("q")}
    bad = {k: v for k, v in keep.items() if not v <= TOL_MIXED}
    assert not bad, f"{name}: {bad}"


# The workloads the benchmark is quoted on, at their own sizes (or half the base mesh):
#  * the Sod tube as configured: 128x4 trees, 2 levels at the jump, 28^2 velocity grid, outflow
#    in x, periodic in y, over its full 100 steps;
#  * the cylinder with its 48^2 velocity roots adapted by 2 levels, at half the base mesh
#    (15.9 M phase cells);
#  * the Sod tube with InterpolatedOutflow ends (CAIDVM.jl:71-94), the linear extrapolation
#    past the domain face.
from kitgpu import mesh as _mesh  # noqa: E402

CONFIG_CASES = [
    ("sod_128x4_L2_v28_100_steps", lambda: cases.sod(), 100),
    ("cylinder_v48_vsL2_half_mesh", lambda: cases.cylinder(scale=0.5, nv=48, vs_levels=2), 2),
    ("sod_interpolated_outflow", lambda: cases.sod(scale=0.25, nv=16, x_bc=_mesh.BC_INTERP), 20),
]


@pytest.mark.parametrize("name,make,nsteps", CONFIG_CASES, ids=[c[0] for c in CONFIG_CASES])
def test_config_fp64_matches_oracle(name, make, nsteps):
    """FP64 within 1e-12 of the oracle on every moment component and on f."""
    topo, ref, out, rep = run_pair(make(), nsteps, check=10)
    errs = moment_errors(topo, ref.w, ref.prim, ref.qf, out["w"], out["prim"], out["qf"])
    errs["f"] = f_error(topo, ref.f, out["f"])
    bad = {k: v for k, v in errs.items() if not v <= TOL_FP64}
    assert not bad, f"{name}: {bad}"


@pytest.mark.parametrize("name,make,nsteps", CONFIG_CASES, ids=[c[0] for c in CONFIG_CASES])
def test_config_mixed_within_1e5_of_oracle(name, make, nsteps):
    """Mixed form within 1e-5 of the FP64 oracle on ρ, U, T and q (the Sod tube over all of
    its 100 steps)."""
    topo, ref, out, rep = run_pair(make(), nsteps, precision=abi.KG_PREC_MIXED, check=10)
    errs = moment_errors(topo, ref.w, ref.prim, ref.qf, out["w"], out["prim"], out["qf"])
    keep = {k: v for k, v in errs.items() if k in ("rho", "T") or k.startswith("U") or k.startswith("q")}
    bad = {k: v for k, v in keep.items() if not v <= TOL_MIXED}
    assert not bad, f"{name}: {bad}"


SW_CASES = [CASES_FP64[1], CASES_FP64[3], CASES_FP64[4]]


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED])
@pytest.mark.parametrize("name,make,nsteps", SW_CASES, ids=[c[0] for c in SW_CASES])
def test_macro_slopes_match_oracle(name, make, nsteps, prec):
    """sw of update_macro_slope! (moments of each direction's slopes) from the slopes the last
    step left.  FP64: 1e-10 of each component's own scale.  Mixed form: a slope is a difference
    of neighbouring f over ds, so the ~1e-6 relative error of FP32-stored f after a few steps
    shows up as ~1e-6 |w| / ds in sw, not relative to sw itself; the mixed form is held to
    1e-5 of max|w_j| / min ds.  Solid cells get zeros."""
    p = make()
    topo, ref, out, _ = run_pair(p, nsteps, precision=prec)
    ref_sw = ref.macro_slope(abi.make_params(p))
    got = out["sw"]
    be = np.asarray(topo["cell_bound_enc"])
    assert np.all(got[be < 0] == 0.0)
    dim = topo["dim"]
    w = ref.w.reshape(-1, dim + 2)[be >= 0]
    vt = float(np.max(np.sqrt(1.0 / ref.prim.reshape(-1, dim + 2)[be >= 0, -1])))
    ds_min = float(np.min(np.asarray(topo["cell_ds"]).reshape(-1, dim)))
    floor = 1e-3 * float(np.max(np.abs(ref_sw)))
    for j in range(dim + 2):
        r, g = ref_sw[be >= 0, :, j], got[be >= 0, :, j]
        if prec == abi.KG_PREC_FP64:
            tol, scale = 1e-10, max(float(np.max(np.abs(r))), floor)
        else:
            # momentum components against ρ v_th (a flow at rest has ρU ~ 0 but not its error)
            mag = float(np.max(np.abs(w[:, j])))
            if 1 <= j <= dim:
                mag = max(mag, float(np.max(np.abs(w[:, 0]))) * vt)
            tol, scale = 1e-5, mag / ds_min
        err = float(np.max(np.abs(g - r))) / scale
        assert err <= tol, (name, j, err)


@pytest.mark.parametrize("name,make,nsteps", [CASES_FP64[1], CASES_FP64[3]], ids=["cavity_levels", "cylinder_ib_adapted"])
def test_downloaded_slopes_match_oracle(name, make, nsteps):
    """sdf after the last step (kg_download_state's sdf): the slopes that step's flux used,
    FP64 within 1e-12 of the largest slope."""
    import oracle as O
    from kitgpu.solver import GpuStep
    p = make()
    topo, state = cases.build(p)
    prm = abi.make_params(p, st_check_interval=1)
    ref = O.OracleState(topo, state).run(prm, p.dt(), 0, nsteps, nthreads=4)
    g = GpuStep(prm, topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    g.step(p.dt(), 0, nsteps)
    out = g.download_state(sdf=True)
    g.close()
    be = np.asarray(topo["cell_bound_enc"])
    from kitgpu import mesh
    off = mesh.f_offsets(topo)
    dim = topo["dim"]
    mask = np.zeros(ref.sdf.size, bool)
    for c in np.nonzero(be >= 0)[0]:
        mask[off[c] * dim:off[c + 1] * dim] = True
    scale = float(np.max(np.abs(ref.sdf[mask])))
    assert float(np.max(np.abs(out["sdf"][mask] - ref.sdf[mask]))) <= 1e-12 * scale


@pytest.mark.parametrize("name,make,nsteps", [CASES_FP64[1], CASES_FP64[3], CASES_FP64[4]],
                         ids=["cavity_levels", "cylinder_ib_adapted", "box3d_levels"])
def test_criterion_matches_oracle(name, make, nsteps):
    """PsData.lohner after the last step (update_criterion! + buffer layer) through
    kg_criterion, against the oracle's restatement on its own state: FP64 within 1e-9."""
    import oracle as O
    from kitgpu.solver import GpuStep
    p = make()
    topo, state = cases.build(p)
    prm = abi.make_params(p, st_check_interval=1)
    ref = O.OracleState(topo, state).run(prm, p.dt(), 0, nsteps, nthreads=4)
    g = GpuStep(prm, topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    g.step(p.dt(), 0, nsteps)
    thr = 0.05
    got = g.criterion(thr)
    sdf = g.download_state(sdf=True)["sdf"]
    g.close()
    exp = ref.criterion(prm, thr)
    assert np.any(exp > 0), "the case exercises the sensor"
    err = np.abs(got - exp)
    assert np.all(err <= 1e-9 * np.maximum(1.0, np.abs(exp))), (name, float(err.max()))
    # the criterion ran on fresh slopes of the current f (slope! before update_criterion!),
    # and they stay on the device
    from kitgpu import mesh
    off, dim = mesh.f_offsets(topo), topo["dim"]
    mask = np.zeros(ref.sdf.size, bool)
    for c in np.nonzero(np.asarray(topo["cell_bound_enc"]) >= 0)[0]:
        mask[off[c] * dim:off[c + 1] * dim] = True
    assert float(np.max(np.abs(sdf[mask] - ref.sdf[mask]))) <= 1e-12 * float(np.max(np.abs(ref.sdf[mask])))


def test_mixed_tracks_fp64_over_200_steps():
    """The mixed form does not drift: 200 steps of the cylinder (walls, adapted velocity grids)
    against the FP64 form, ρ, U, T and q within 1e-5 (measured: ~1e-7 after 500 steps)."""
    from kitgpu.solver import GpuStep
    from parity import moment_errors
    p = cases.cylinder(scale=0.25, nv=24, vs_levels=2)
    topo, state = cases.build(p)
    out = {}
    for prec in (abi.KG_PREC_FP64, abi.KG_PREC_MIXED):
        g = GpuStep(abi.make_params(p, precision=prec, st_check_interval=1), topo)
        g.upload_state(state["f"], state["w"], state["prim"])
        g.step(p.dt(), 0, 200)
        out[prec] = g.download_state()
        g.close()
    a, b = out[abi.KG_PREC_FP64], out[abi.KG_PREC_MIXED]
    errs = moment_errors(topo, a["w"], a["prim"], a["qf"], b["w"], b["prim"], b["qf"])
    keep = {k: v for k, v in errs.items() if k in ("rho", "T") or k[0] in "Uq"}
    assert all(v <= TOL_MIXED for v in keep.values()), keep
