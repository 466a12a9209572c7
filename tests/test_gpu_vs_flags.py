"""Velocity-space adaptation flags on the device (kg_vs_flags): the per-velocity decisions of
vs_refine! / vs_coarsen! against the oracle's restatement (which locates face neighbours with
the reference's own sorted-key index)."""
import numpy as np
import pytest

from kitgpu import abi, cases

pytestmark = pytest.mark.gpu

VS_CASES = [
    ("cylinder_vs_adapted", lambda: cases.cylinder(scale=0.25, nv=24, vs_levels=2), 3),
    ("collision_two_grids", lambda: cases.collision(center=0.5), 3),
    ("box3d", lambda: cases.box3d(n=(6, 4, 4), nv=8, levels=1), 2),
    ("sphere3d_ib", lambda: cases.sphere(scale=0.25, nv=8), 2),
]


def _states(make, nsteps, prec):
    import oracle as O
    from kitgpu.solver import GpuStep
    p = make()
    topo, state = cases.build(p)
    prm64 = abi.make_params(p, st_check_interval=1)
    ref = O.OracleState(topo, state).run(prm64, p.dt(), 0, nsteps, nthreads=4)
    g = GpuStep(abi.make_params(p, precision=prec, st_check_interval=1), topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    g.step(p.dt(), 0, nsteps)
    return p, prm64, ref, g


@pytest.mark.parametrize("mode", [abi.KG_VS_LOHNER, abi.KG_VS_CONTRIBUTION], ids=["lohner", "contribution"])
@pytest.mark.parametrize("name,make,nsteps", VS_CASES, ids=[c[0] for c in VS_CASES])
def test_vs_flags_fp64_match_oracle(name, make, nsteps, mode):
    p, prm64, ref, g = _states(make, nsteps, abi.KG_PREC_FP64)
    maxlevel = max(p.vs_maxlevel, 1)
    cfg = abi.make_vs_config(p, maxlevel=maxlevel, mode=mode)
    fl, eta, vr = g.vs_flags(cfg)
    g.close()
    efl, eeta, evr = ref.vs_flags(prm64, cfg)
    assert fl.size == efl.size
    assert np.allclose(vr, evr, rtol=1e-12, atol=0)
    assert np.any(efl & 1) and np.any(efl & 2), "the case exercises both flags"
    assert np.max(np.abs(eta - eeta)) <= 1e-12 * max(1.0, float(np.max(np.abs(eeta))))
    # flags are threshold decisions on values equal to rounding: all equal here
    assert np.array_equal(fl, efl), (name, int(np.sum(fl != efl)))


def test_vs_flags_mixed_close_to_fp64():
    p, prm64, ref, g = _states(VS_CASES[0][1], 3, abi.KG_PREC_MIXED)
    cfg = abi.make_vs_config(p)
    fl, eta, vr = g.vs_flags(cfg)
    g.close()
    efl, eeta, evr = ref.vs_flags(prm64, cfg)
    assert np.allclose(vr, evr, rtol=1e-5)
    assert np.max(np.abs(eta - eeta)) <= 1e-4
    # f is stored in FP32: a decision can flip only where the FP64 value sits at a threshold
    assert np.mean(fl != efl) < 1e-3


def test_batch_vs_flags_equal_single():
    from kitgpu.solver import GpuBatch
    p, prm64, ref, g = _states(VS_CASES[1][1], 2, abi.KG_PREC_FP64)
    cfg = abi.make_vs_config(p)
    fl, eta, vr = g.vs_flags(cfg)
    g.close()
    topo, state = cases.build(p)
    q = cases.cavity(n=8, nv=12)
    tq, sq = cases.build(q)
    prm = abi.make_params(p, st_check_interval=1)
    b = GpuBatch(prm, pool_bytes=64 << 20)
    b.admit(abi.make_params(q, st_check_interval=1), tq, sq["f"], sq["w"], sq["prim"], q.dt())
    s1 = b.admit(prm, topo, state["f"], state["w"], state["prim"], p.dt())
    b.step(2)
    bfl, beta, bvr = b.vs_flags(s1, cfg)
    b.close()
    assert np.array_equal(bfl, fl) and np.array_equal(beta, eta) and np.array_equal(bvr, vr)
