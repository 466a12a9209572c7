"""Batched form: independent problems of uneven cell/velocity counts and their own gas
constants advance together; each result must be bitwise the same alone and in the mix,
also across admissions and releases and under CUDA-graph replay."""
import numpy as np
import pytest

from kitgpu import abi, cases
from kitgpu.solver import GpuBatch, GpuStep, KitGpuError

pytestmark = pytest.mark.gpu


def _problems():
    return [cases.sod(scale=0.125, nv=16), cases.cavity(n=8, nv=12, levels=1, Kn=0.01),
            cases.cylinder(scale=0.125, nv=16, vs_levels=1), cases.couette(n=6, nv=20)]


def _alone(problem, topo, state, prec, nsteps):
    g = GpuStep(abi.make_params(problem, precision=prec, st_check_interval=2), topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    rep = g.step(problem.dt(), 0, nsteps)
    out = g.download_state()
    g.close()
    return out, rep


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_results_equal_alone(prec, graph):
    probs = _problems()
    built = [cases.build(p) for p in probs]
    b = GpuBatch(abi.make_params(probs[0], precision=prec), 512 << 20)
    if graph:
        b.use_graph(True)
    slots = []
    for p, (t, s) in zip(probs[:3], built[:3]):
        slots.append(b.admit(abi.make_params(p, precision=prec, st_check_interval=2), t, s["f"], s["w"], s["prim"], p.dt()))
    reps = b.step(2)
    reps = b.step(2)
    for k in range(3):
        ref, rrep = _alone(probs[k], built[k][0], built[k][1], prec, 4)
        got = b.download(slots[k])
        for key in ("f", "w", "prim", "qf"):
            assert np.array_equal(got[key], ref[key]), (k, key)
        assert reps[slots[k]].checked and rrep.checked
        nw = built[k][0]["dim"] + 2
        assert np.array_equal(np.array(reps[slots[k]].sum_res[:nw]), np.array(rrep.sum_res[:nw]))
    # membership change: release the first, admit the fourth, continue
    b.release(slots[0])
    p3, (t3, s3) = probs[3], built[3]
    s_new = b.admit(abi.make_params(p3, precision=prec, st_check_interval=2), t3, s3["f"], s3["w"], s3["prim"], p3.dt())
    b.step(3)
    ref3, _ = _alone(p3, t3, s3, prec, 3)
    assert np.array_equal(b.download(s_new)["f"], ref3["f"])
    ref1, _ = _alone(probs[1], built[1][0], built[1][1], prec, 7)
    assert np.array_equal(b.download(slots[1])["f"], ref1["f"])
    b.close()


def test_batch_refuses_over_budget():
    p = cases.sod(scale=0.125, nv=16)
    t, s = cases.build(p)
    b = GpuBatch(abi.make_params(p), 8 << 20)     # 8 MiB: room for one small problem
    b.admit(abi.make_params(p), t, s["f"], s["w"], s["prim"], p.dt())
    with pytest.raises(KitGpuError) as e:
        for _ in range(64):
            b.admit(abi.make_params(p), t, s["f"], s["w"], s["prim"], p.dt())
    assert e.value.code == 8   # KG_ERR_BUDGET
    b.close()


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED])
def test_autotuned_persistent_schedule_gives_same_results(prec):
    probs = _problems()
    built = [cases.build(p) for p in probs]
    outs = []
    for tune in (False, True):
        b = GpuBatch(abi.make_params(probs[0], precision=prec), 512 << 20)
        b.autotune(tune)
        slots = [b.admit(abi.make_params(p, precision=prec, st_check_interval=2), t, s["f"], s["w"], s["prim"], p.dt())
                 for p, (t, s) in zip(probs, built)]
        b.step(3)
        res = b.autotune_result()
        if tune:
            assert len(res["trial_ms"]) >= 3
        outs.append([b.download(sl) for sl in slots])
        b.close()
    for a, c in zip(outs[0], outs[1]):
        for key in ("f", "w", "prim", "qf"):
            assert np.array_equal(a[key], c[key])


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED])
def test_large_pool_admission_keeps_state(prec):
    """A pool of about half the device: its zero fill takes tens of ms, and an admission
    right after creating the batch must still find its state intact (the fill and the
    upload run in order on the handle's stream) and step like the problem alone."""
    import torch
    free = torch.cuda.mem_get_info()[0]
    p = cases.cavity(n=8, nv=12, levels=0, Kn=0.3)
    t, s = cases.build(p)
    b = GpuBatch(abi.make_params(p, precision=prec), int(min(free * 0.5, 160 << 30)))
    slot = b.admit(abi.make_params(p, precision=prec, st_check_interval=2), t, s["f"], s["w"], s["prim"], p.dt())
    got = b.download(slot)
    assert np.array_equal(got["w"], s["w"]) and np.array_equal(got["prim"], s["prim"])
    if prec == abi.KG_PREC_FP64:
        assert np.array_equal(got["f"], s["f"])
    else:
        assert np.array_equal(got["f"], s["f"].astype(np.float32).astype(np.float64))
    b.step(2)
    ref, _ = _alone(p, t, s, prec, 2)
    assert np.array_equal(b.download(slot)["f"], ref["f"])
    b.close()


def test_batch_sw_equals_single_handle():
    """kg_batch_download_sw of a problem in a batch is bitwise kg_download_sw of it alone."""
    probs = _problems()[:2]
    built = [cases.build(p) for p in probs]
    prec = abi.KG_PREC_MIXED
    b = GpuBatch(abi.make_params(probs[0], precision=prec), 512 << 20)
    slots = [b.admit(abi.make_params(p, precision=prec, st_check_interval=2), t, s["f"], s["w"], s["prim"], p.dt())
             for p, (t, s) in zip(probs, built)]
    b.step(3)
    for k, (p, (t, s)) in enumerate(zip(probs, built)):
        g = GpuStep(abi.make_params(p, precision=prec, st_check_interval=2), t)
        g.upload_state(s["f"], s["w"], s["prim"])
        g.step(p.dt(), 0, 3)
        assert np.array_equal(b.download_sw(slots[k]), g.download_sw())
        g.close()
    b.close()


def test_batch_criterion_equals_single_handle():
    probs = _problems()[:3]
    built = [cases.build(p) for p in probs]
    prec = abi.KG_PREC_MIXED
    b = GpuBatch(abi.make_params(probs[0], precision=prec), 512 << 20)
    slots = [b.admit(abi.make_params(p, precision=prec, st_check_interval=2), t, s["f"], s["w"], s["prim"], p.dt())
             for p, (t, s) in zip(probs, built)]
    b.step(2)
    for k, (p, (t, s)) in enumerate(zip(probs, built)):
        g = GpuStep(abi.make_params(p, precision=prec, st_check_interval=2), t)
        g.upload_state(s["f"], s["w"], s["prim"])
        g.step(p.dt(), 0, 2)
        assert np.array_equal(b.criterion(slots[k], 0.05), g.criterion(0.05))
        g.close()
    b.close()
