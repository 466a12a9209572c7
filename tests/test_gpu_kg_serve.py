"""kg_serve: pipelined requests (upload of the next and download of the previous request on
copy streams while one steps) give, bit for bit, the results of upload + step + download."""
import numpy as np
import pytest

from kitgpu import abi, cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name,make", [
    ("sod", lambda: cases.sod(scale=0.125, nv=16)),
    ("cylinder_ib", lambda: cases.cylinder(scale=0.25, nv=16, vs_levels=1)),
])
def test_serve_equals_upload_step_download(name, make, prec):
    from kitgpu.solver import GpuStep
    p = make()
    topo, state = cases.build(p)
    nw = topo["dim"] + 2
    reqs = []
    for r in range(3):
        s = 1.0 + 0.01 * r
        prim = state["prim"].copy().reshape(-1, nw)
        prim[:, 0] *= s   # density scaled with f and w: velocity and temperature unchanged
        reqs.append({"f": state["f"] * s, "w": state["w"] * s, "prim": prim.ravel()})
    prm = abi.make_params(p, precision=prec, st_check_interval=2)
    dt, nsteps, step0 = p.dt(), 3, 4
    g = GpuStep(prm, topo)
    g.upload_state(state["f"], state["w"], state["prim"])   # any state: serve replaces it
    outs, reps = g.serve(reqs, dt, step0, nsteps)
    last = g.download_state()
    g.close()
    for r, st in enumerate(reqs):
        h = GpuStep(prm, topo)
        h.upload_state(st["f"], st["w"], st["prim"])
        rep = h.step(dt, step0, nsteps)
        ref = h.download_state()
        h.close()
        for k in ("f", "w", "prim", "qf"):
            assert np.array_equal(outs[r][k], ref[k]), (name, r, k)
        assert reps[r].checked == rep.checked and reps[r].checked_step == rep.checked_step
        assert np.array_equal(np.array(reps[r].sum_res[:nw]), np.array(rep.sum_res[:nw]))
        assert reps[r].status == 0 and reps[r].kernel_launches == rep.kernel_launches
    for k in ("f", "w", "prim", "qf"):
        assert np.array_equal(last[k], outs[-1][k])
