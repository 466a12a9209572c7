"""Physical-space adaptation on the device (kg_adapt / kg_batch_adapt, the state moves of
ps_replace!) against the oracle's restatement: the interpolated state, and the steps that
follow it on the adapted mesh."""
import numpy as np
import pytest

from kitgpu import abi, cases, mesh
from parity import TOL_FP64, TOL_MIXED, f_error, moment_errors

pytestmark = pytest.mark.gpu


def _meshes(make_old, make_new):
    pa, pb = make_old(), make_new()
    ta, sa = cases.build(pa)
    tb, _ = cases.build(pb)
    src = mesh.adapt_sources(ta, tb)
    tb = mesh.adapt_grids(ta, tb, src)
    return pa, ta, sa, tb, src


def _sdf_error(topo, ref, got):
    off, dim = mesh.f_offsets(topo), topo["dim"]
    mask = np.zeros(ref.size, bool)
    for c in np.nonzero(np.asarray(topo["cell_bound_enc"]) >= 0)[0]:
        mask[off[c] * dim:off[c + 1] * dim] = True
    return float(np.max(np.abs(got[mask] - ref[mask]))) / float(np.max(np.abs(ref[mask])))


def _check_state(topo, ref, out, tol, sdf=True):
    errs = moment_errors(topo, ref.w, ref.prim, ref.qf, out["w"], out["prim"], out["qf"])
    errs["f"] = f_error(topo, ref.f, out["f"])
    if sdf:
        errs["sdf"] = _sdf_error(topo, ref.sdf, out["sdf"])
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, bad


ADAPT_CASES = [
    ("collision_2grids", lambda: cases.collision(center=0.5), lambda: cases.collision(center=0.62)),
    ("collision_back", lambda: cases.collision(center=0.62), lambda: cases.collision(center=0.5)),
    ("box3d", lambda: cases.box3d(n=(6, 4, 4), nv=8, levels=1),
     lambda: _box3d_shift()),
    ("cylinder_far_field", lambda: cases.cylinder(scale=0.125, max_level=2, nv=16, vs_levels=0),
     lambda: _cylinder_extra()),
]


def _box3d_shift():
    p = cases.box3d(n=(6, 4, 4), nv=8, levels=1)
    p.case.refine = lambda mid, ds, L: abs(mid[0] - 0.62) < 1.2 * ds[0]
    return p


def _cylinder_extra():
    # the wall region as before (walls, solid and donor cells kept), a refined band far
    # downstream and the outer ring coarsened upstream
    p = cases.cylinder(scale=0.125, max_level=2, nv=16, vs_levels=0)
    base = p.case.refine

    def refine(mid, ds, L):
        if L == 0 and mid[0] > 5.5 and abs(mid[1]) < 3.5:
            return True
        if L == 1 and mid[0] < -2.5:
            return False
        return base(mid, ds, L)
    p.case.refine = refine
    return p


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name,make_old,make_new", ADAPT_CASES, ids=[c[0] for c in ADAPT_CASES])
def test_adapt_matches_oracle(name, make_old, make_new, prec):
    import oracle as O
    from kitgpu.solver import GpuStep
    pa, ta, sa, tb, src = _meshes(make_old, make_new)
    kinds = np.bincount(src["kind"], minlength=3)
    assert kinds[abi.KG_ADAPT_REFINE] > 0 and (kinds[abi.KG_ADAPT_COARSEN] > 0 or name.startswith("cylinder"))
    prm64 = abi.make_params(pa, st_check_interval=1)
    prm = abi.make_params(pa, precision=prec, st_check_interval=1)
    dt = pa.dt()
    ref = O.OracleState(ta, sa).run(prm64, dt, 0, 3, nthreads=4)
    g = GpuStep(prm, ta)
    g.upload_state(sa["f"], sa["w"], sa["prim"])
    g.step(dt, 0, 3)
    g.adapt(tb, src)
    out = g.download_state(sdf=True)
    ref2 = ref.adapt(prm64, tb, src)
    tol = TOL_FP64 if prec == abi.KG_PREC_FP64 else TOL_MIXED
    _check_state(tb, ref2, out, tol)
    # the adapted mesh steps on (walls restarted from their donors, as after amr_recover!)
    ref2.run(prm64, dt, 3, 3, nthreads=4)
    g.step(dt, 3, 3)
    out = g.download_state()
    g.close()
    _check_state(tb, ref2, out, tol, sdf=False)


def test_adapt_refine_all_then_coarsen_back_is_the_identity():
    """Size-independent property on the full Sod tube: one level everywhere, then back.  The
    children's offsets cancel (one limiter per velocity cell), so f returns to rounding."""
    from kitgpu.solver import GpuStep
    p = cases.sod(scale=1.0, max_level=0)
    ta, sa = cases.build(p)
    p2 = cases.sod(scale=1.0, max_level=0)
    p2.case.max_level, p2.case.refine = 1, (lambda mid, ds, L: True)
    tb, _ = cases.build(p2)
    fwd = mesh.adapt_sources(ta, tb)
    back = mesh.adapt_sources(tb, ta)
    assert np.all(fwd["kind"] == abi.KG_ADAPT_REFINE) and np.all(back["kind"] == abi.KG_ADAPT_COARSEN)
    for prec, tol in ((abi.KG_PREC_FP64, 1e-14), (abi.KG_PREC_MIXED, 2e-7)):
        g = GpuStep(abi.make_params(p, precision=prec), ta)
        g.upload_state(sa["f"], sa["w"], sa["prim"])
        g.step(p.dt(), 0, 5)
        before = g.download_state()
        g.adapt(tb, fwd)
        mid = g.download_state()
        assert mid["f"].size == 4 * before["f"].size
        g.adapt(ta, back)
        after = g.download_state()
        g.close()
        assert np.max(np.abs(after["f"] - before["f"])) <= tol * np.max(np.abs(before["f"])), prec
        assert np.max(np.abs(mid["f"] - np.repeat(before["f"].reshape(ta["n_cells"], -1), 4, axis=0).reshape(-1))) > 0


def test_adapt_rejects_a_bad_plan_and_keeps_the_mesh():
    import oracle as O
    from kitgpu.solver import GpuStep, KitGpuError
    pa, ta, sa, tb, src = _meshes(lambda: cases.collision(center=0.5), lambda: cases.collision(center=0.62))
    prm = abi.make_params(pa, st_check_interval=1)
    g = GpuStep(prm, ta)
    g.upload_state(sa["f"], sa["w"], sa["prim"])
    g.step(pa.dt(), 0, 2)
    r = int(np.nonzero(src["kind"] == abi.KG_ADAPT_REFINE)[0][0])
    bad = src.copy()
    bad[r]["depth"] = 0                          # a refinement of depth 0
    with pytest.raises(KitGpuError) as e:
        g.adapt(tb, bad)
    assert e.value.code == 1                     # KG_ERR_ARG
    bad = src.copy()
    bad[r]["src"][0] = ta["n_cells"]             # a source out of range
    with pytest.raises(KitGpuError) as e:
        g.adapt(tb, bad)
    assert e.value.code == 1
    c = int(np.nonzero(src["kind"] == abi.KG_ADAPT_COARSEN)[0][0])
    grids = tb["cell_grid"].copy()
    tb_bad = dict(tb, cell_grid=grids)
    ch = src[c]["src"][:4]
    alt = [g_ for g_ in set(ta["cell_grid"].tolist()) if g_ != grids[c]]
    grids[c] = alt[0]                            # not the grid ps_merge keeps
    with pytest.raises(KitGpuError) as e:
        g.adapt(tb_bad, src)
    assert e.value.code == 2                     # KG_ERR_TOPOLOGY
    assert len(set(ta["cell_grid"][ch].tolist())) >= 1
    # the handle still holds the previous mesh and state
    ref = O.OracleState(ta, sa).run(prm, pa.dt(), 0, 4, nthreads=4)
    g.step(pa.dt(), 2, 2)
    out = g.download_state()
    g.close()
    _check_state(ta, ref, out, TOL_FP64, sdf=False)


def test_batch_adapt_matches_single():
    from kitgpu.solver import GpuBatch, GpuStep
    pa, ta, sa, tb, src = _meshes(lambda: cases.collision(center=0.5), lambda: cases.collision(center=0.62))
    pc = cases.cavity(n=8, nv=12)
    tc, sc = cases.build(pc)
    prm = abi.make_params(pa, st_check_interval=1)
    prmc = abi.make_params(pc, st_check_interval=1)
    dt = pa.dt()
    single = GpuStep(prm, ta)
    single.upload_state(sa["f"], sa["w"], sa["prim"])
    single.step(dt, 0, 3)
    single.adapt(tb, src)
    single.step(dt, 3, 2)
    exp = single.download_state()
    single.close()
    solo_c = GpuStep(prmc, tc)
    solo_c.upload_state(sc["f"], sc["w"], sc["prim"])
    solo_c.step(pc.dt(), 0, 5)
    exp_c = solo_c.download_state()
    solo_c.close()
    b = GpuBatch(prm, pool_bytes=64 << 20)
    s0 = b.admit(prm, ta, sa["f"], sa["w"], sa["prim"], dt)
    s1 = b.admit(prmc, tc, sc["f"], sc["w"], sc["prim"], pc.dt())
    b.step(3)
    b.adapt(s0, tb, src)
    b.step(2)
    got, got_c = b.download(s0), b.download(s1)
    b.close()
    for k in ("f", "w", "prim"):
        assert np.array_equal(got[k], exp[k]), k
        assert np.array_equal(got_c[k], exp_c[k]), k
