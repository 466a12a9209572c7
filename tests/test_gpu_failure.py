"""Failure detection through the device status words, with the failure made on the host.

A state with one bad cell is uploaded (a NaN in one velocity cell's f, or a negative density
in one cell's conserved variables); the kernels flag the cell's primitive variables and
kg_step returns KG_ERR_NONFINITE / KG_ERR_NEGATIVE.  In a batch only the problem that holds
the bad cell is flagged, and the other problems' results are bitwise those of a clean run.
Nothing here faults or stalls the GPU: the kernels only set status bits, and the context
stays usable for the next call."""
import ctypes as C

import numpy as np
import pytest

from kitgpu import abi, cases, mesh
from kitgpu.solver import MAX_SLOTS, GpuBatch, GpuStep, KitGpuError

pytestmark = pytest.mark.gpu

KG_ERR_NONFINITE, KG_ERR_NEGATIVE = 5, 6


def _fluid_cell(topo, which=0.5):
    fluid = np.nonzero(np.asarray(topo["cell_bound_enc"]) >= 0)[0]
    return int(fluid[int(which * (len(fluid) - 1))])


def _nan_state(topo, state):
    st = {k: v.copy() for k, v in state.items()}
    c = _fluid_cell(topo)
    off = mesh.f_offsets(topo)
    st["f"][off[c] + 3] = np.nan
    return st


def _negative_state(topo, state):
    st = {k: v.copy() for k, v in state.items()}
    c = _fluid_cell(topo)
    nw = topo["dim"] + 2
    st["w"][c * nw] = -abs(st["w"][c * nw])
    return st


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED])
@pytest.mark.parametrize("kind,make,code", [("nan", _nan_state, KG_ERR_NONFINITE),
                                            ("negative", _negative_state, KG_ERR_NEGATIVE)])
def test_step_reports_bad_state(prec, kind, make, code):
    p = cases.sod(scale=0.125, nv=16)
    topo, state = cases.build(p)
    bad = make(topo, state)
    g = GpuStep(abi.make_params(p, precision=prec, st_check_interval=1), topo)
    g.upload_state(bad["f"], bad["w"], bad["prim"])
    with pytest.raises(KitGpuError) as ei:
        g.step(p.dt(), 0, 1)
    assert ei.value.code == code, (kind, ei.value)
    # the handle and the context stay usable: a clean state steps without error afterwards
    # (an upload resets the status word)
    g.upload_state(state["f"], state["w"], state["prim"])
    rep = g.step(p.dt(), 0, 2)
    assert rep.status == 0
    out = g.download_state()
    g.close()
    assert np.all(np.isfinite(out["f"]))


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED])
def test_batch_flags_only_the_bad_problem(prec):
    probs = [cases.sod(scale=0.125, nv=16), cases.cavity(n=8, nv=12, levels=1), cases.sod(scale=0.125, nv=12)]
    built = [cases.build(q) for q in probs]
    b = GpuBatch(abi.make_params(probs[0], precision=prec), 256 << 20)
    slots = []
    for k, (q, (t, s)) in enumerate(zip(probs, built)):
        st = _nan_state(t, s) if k == 1 else s
        slots.append(b.admit(abi.make_params(q, precision=prec, st_check_interval=1), t, st["f"], st["w"], st["prim"],
                             q.dt()))
    reports = (abi.KgStepReport * MAX_SLOTS)()
    rc = b.L.kg_batch_step(b.h, 2, reports, MAX_SLOTS)
    assert rc == KG_ERR_NONFINITE
    assert reports[slots[1]].status == KG_ERR_NONFINITE
    assert reports[slots[0]].status == 0 and reports[slots[2]].status == 0
    # the clean problems advanced exactly as they would alone
    for k in (0, 2):
        q, (t, s) = probs[k], built[k]
        g = GpuStep(abi.make_params(q, precision=prec, st_check_interval=1), t)
        g.upload_state(s["f"], s["w"], s["prim"])
        g.step(q.dt(), 0, 2)
        ref = g.download_state()
        g.close()
        got = b.download(slots[k])
        for key in ("f", "w", "prim", "qf"):
            assert np.array_equal(got[key], ref[key]), (k, key)
    # releasing the bad problem leaves a batch that steps cleanly
    b.release(slots[1])
    b.step(1)
    b.close()
