"""Velocity-space adaptation on the device: kg_adapt with KG_ADAPT_VS records moves f onto
grids rebuilt by refine_grid_stream! / coarsen_grid_stream! (Velocity_space/Rebuild.jl:44-163)
and kg_vs_conserve corrects them (vs_conserved_correction!), against the oracle."""
import numpy as np
import pytest

import oracle as O
from kitgpu import abi, cases, mesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name,make", [
    ("sod_levels", lambda: cases.sod(scale=0.125, nv=16)),
    ("box3d", lambda: cases.box3d(n=(6, 4, 4), nv=8, levels=1)),
])
def test_vs_refine_coarsen_on_device(name, make, prec):
    from kitgpu.solver import GpuStep
    p = make()
    topo, state = cases.build(p)
    dim = topo["dim"]
    prm = abi.make_params(p, precision=prec)
    prm64 = abi.make_params(p)
    dt = p.dt()
    g = GpuStep(prm, topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    g.step(dt, 0, 2)
    s0 = g.download_state()
    root = mesh.vgrid_root_ds(p.case.quadrature, p.case.vs_trees_num, dim)
    fine = {}
    for c in range(0, topo["n_cells"], 2):
        vg = mesh.cell_vgrid(topo, c)
        fine[c] = mesh.refine_vgrid(vg, np.linalg.norm(vg.midpoint, axis=1) < 2.0, root)
    t1 = mesh.with_cell_vgrids(topo, fine)
    g.adapt(t1, mesh.vs_sources(t1))
    s1 = g.download_state(sdf=True)
    ref = O.OracleState(topo, dict(f=s0["f"], w=s0["w"], prim=s0["prim"]))
    ref.qf[:] = s0["qf"]
    r1 = ref.adapt(prm64, t1, mesh.vs_sources(t1))
    tol = 0.0 if prec == abi.KG_PREC_FP64 else 1e-6
    err = float(np.max(np.abs(s1["f"] - r1.f)) / np.max(np.abs(r1.f)))
    assert err <= tol, (name, err)
    assert np.all(s1["sdf"] == 0.0)
    assert np.array_equal(s1["w"], s0["w"]) and np.array_equal(s1["prim"], s0["prim"])
    # the conservative correction of the changed cells, then coarsening back
    flags = np.zeros(topo["n_cells"], np.uint8)
    flags[list(fine)] = 1
    g.vs_conserve(flags)
    coarse = {c: mesh.coarsen_vgrid(mesh.cell_vgrid(t1, c), mesh.cell_vgrid(t1, c).level > 0, root, 2) for c in fine}
    t2 = mesh.with_cell_vgrids(t1, coarse)
    g.adapt(t2, mesh.vs_sources(t2))
    g.vs_conserve(flags)
    s2 = g.download_state()
    # the steps go on from the adapted state as the oracle's do from the same state
    rep = g.step(dt, 2, 2)
    out = g.download_state()
    g.close()
    assert rep.status == 0
    st = O.OracleState(t2, dict(f=s2["f"], w=s2["w"], prim=s2["prim"]))
    st.run(prm64, dt, 2, 2)
    err = float(np.max(np.abs(out["f"] - st.f)) / np.max(np.abs(st.f)))
    assert err <= (1e-12 if prec == abi.KG_PREC_FP64 else 1e-5), (name, err)
