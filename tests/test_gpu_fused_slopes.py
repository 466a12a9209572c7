"""Slopes computed in the flux kernel (kg_fuse_slopes, the 2D mixed form): the regular cells
whose neighbours are regular compute their slopes and their upwind neighbours' from f with
the slope passes' arithmetic, and the slopes no other cell reads leave the passes.  Results
are the same bits as with every slope in the passes and sdf, and the slopes a call reads back
(kg_download_state's sdf, kg_download_sw) are the last step's, filled in on demand."""
import numpy as np
import pytest

from kitgpu import abi, cases
from kitgpu.solver import GpuBatch, GpuStep

pytestmark = pytest.mark.gpu

CASES = [
    ("cylinder", lambda: cases.cylinder(scale=0.25, nv=16, vs_levels=1), 4),
    ("sod", lambda: cases.sod(scale=0.25, nv=16), 5),
    ("cavity_levels", lambda: cases.cavity(n=12, nv=12, levels=1), 4),
]


def _run(p, topo, state, fuse, nsteps, graph=False):
    g = GpuStep(abi.make_params(p, precision=abi.KG_PREC_MIXED, st_check_interval=1), topo)
    g.fuse_slopes(fuse)
    if graph:
        g.use_graph(True)
    g.upload_state(state["f"], state["w"], state["prim"])
    g.step(p.dt(), 0, nsteps - 1)
    g.step(p.dt(), nsteps - 1, 1)
    out = g.download_state(sdf=True)
    out["sw"] = g.download_sw()
    g.close()
    return out


@pytest.mark.parametrize("name,make,nsteps", CASES, ids=[c[0] for c in CASES])
def test_fused_slopes_give_the_same_bits(name, make, nsteps):
    p = make()
    topo, state = cases.build(p)
    a = _run(p, topo, state, True, nsteps)
    b = _run(p, topo, state, False, nsteps)
    c = _run(p, topo, state, True, nsteps, graph=True)
    for key in ("f", "w", "prim", "qf", "sdf", "sw"):
        assert np.array_equal(a[key], b[key]), (name, key)
        assert np.array_equal(c[key], b[key]), (name, key, "graph")


def test_batch_with_fused_slopes_equals_alone_across_release():
    """A batch whose membership changes between steps keeps every problem's bits (the lazy
    slopes complete under the layout that owns them before it changes)."""
    probs = [cases.sod(scale=0.25, nv=16), cases.cavity(n=10, nv=12, levels=1), cases.sod(scale=0.125, nv=12)]
    built = [cases.build(q) for q in probs]
    b = GpuBatch(abi.make_params(probs[0], precision=abi.KG_PREC_MIXED), 256 << 20)
    slots = [b.admit(abi.make_params(q, precision=abi.KG_PREC_MIXED, st_check_interval=1), t, s["f"], s["w"], s["prim"],
                     q.dt()) for q, (t, s) in zip(probs[:2], built[:2])]
    b.step(3)
    b.release(slots[0])
    q2, (t2, s2) = probs[2], built[2]
    s_new = b.admit(abi.make_params(q2, precision=abi.KG_PREC_MIXED, st_check_interval=1), t2, s2["f"], s2["w"],
                    s2["prim"], q2.dt())
    b.step(2)
    sw = b.download_sw(slots[1])
    got = b.download(slots[1])
    b.close()
    g = GpuStep(abi.make_params(probs[1], precision=abi.KG_PREC_MIXED, st_check_interval=1), built[1][0])
    g.fuse_slopes(False)
    g.upload_state(built[1][1]["f"], built[1][1]["w"], built[1][1]["prim"])
    g.step(probs[1].dt(), 0, 5)
    ref = g.download_state()
    ref_sw = g.download_sw()
    g.close()
    for key in ("f", "w", "prim", "qf"):
        assert np.array_equal(got[key], ref[key]), key
    assert np.array_equal(sw, ref_sw)
    del s_new
