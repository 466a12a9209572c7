"""The gather form built on the device (kg_devflat.cu) equals the host builder's
(kg_flatten.cpp) byte for byte: after a topology upload, under the slope fusion, and after an
adaptation (kg_adapt, amr_recover!'s rebuild of faces and neighbours, Solver/AMR.jl:54-70);
and a handle stepping on the device-built layout gives the same bits as one on the host's."""
import numpy as np
import pytest

from kitgpu import abi, cases, mesh

pytestmark = pytest.mark.gpu

NAMES = ["slope_ops", "slope_nbr", "cell_slope_op", "pass_cells", "screc", "crit_ops", "crit_nbr", "inc_off",
         "inc", "bc_prim", "bc_hl", "fluid_cells", "fluid_reg", "fcrec", "regrec", "r2rec", "slope_items",
         "reg_list", "nonreg_list", "r2_list", "inner_list", "innerp_list", "p_off", "p_j0", "p_cnt", "ib_nbr", "wall_ops", "solid_ops"]

LAYOUTS = [
    ("sod_levels", lambda: cases.sod(scale=0.125, nv=16)),
    ("sod_interp_outflow", lambda: cases.sod(scale=0.125, nv=16, x_bc=mesh.BC_INTERP)),
    ("cavity_levels", lambda: cases.cavity(n=8, nv=16, levels=2)),
    ("couette", lambda: cases.couette(n=12, nv=16)),
    ("collision_2grids", lambda: cases.collision(center=0.5)),
    ("cylinder_ib_adapted", lambda: cases.cylinder(scale=0.25, nv=24, vs_levels=2)),
    ("box3d_levels", lambda: cases.box3d(n=(6, 4, 4), nv=8, levels=1)),
    ("sphere3d_ib", lambda: cases.sphere(scale=0.25, nv=8)),
]


def _pair(prob, topo, state, prec, fuse=False):
    from kitgpu.solver import GpuStep
    prm = abi.make_params(prob, precision=prec, st_check_interval=1)
    out = []
    for dev in (True, False):
        g = GpuStep(prm, topo, device_flatten=dev)
        g.fuse_slopes(fuse)
        g.upload_state(state["f"], state["w"], state["prim"])
        out.append(g)
    return out


# record sizes (bytes) of the arrays of structs, for the first differing record in a message
RECORD = {"slope_ops": 40, "slope_nbr": 8, "screc": 136, "crit_ops": 40, "inc": 208, "fcrec": 80, "regrec": 216,
          "r2rec": 208, "ib_nbr": 8, "wall_ops": 184, "solid_ops": 16}


def _first_diff(nm, x, y):
    if len(x) != len(y):
        return f"{nm}: {len(x)} bytes (device) vs {len(y)} (host)"
    i = next(k for k in range(len(x)) if x[k] != y[k])
    r = RECORD.get(nm, 4)
    return f"{nm}: first difference at byte {i} (record {i // r}, byte {i % r} of {r})"


def _same_layout(a, b, tag):
    msgs = []
    for nm in NAMES:
        x, y = a.layout_read(nm), b.layout_read(nm)
        if x != y:
            msgs.append(_first_diff(nm, x, y))
    assert not msgs, f"{tag}: device and host layouts differ: " + "; ".join(msgs)


def _same_state(a, b, tag):
    x, y = a.download_state(sdf=True), b.download_state(sdf=True)
    for k in ("f", "w", "prim", "qf", "sdf"):
        assert np.array_equal(x[k], y[k], equal_nan=True), f"{tag}: {k} differs"


@pytest.mark.parametrize("name,make", LAYOUTS, ids=[c[0] for c in LAYOUTS])
def test_device_layout_equals_host(name, make):
    p = make()
    topo, state = cases.build(p)
    prec = abi.KG_PREC_MIXED if topo["dim"] == 2 else abi.KG_PREC_FP64
    a, b = _pair(p, topo, state, prec)
    _same_layout(a, b, name)
    for g in (a, b):
        g.step(p.dt(), 0, 3)
    _same_state(a, b, name)
    a.close()
    b.close()


@pytest.mark.parametrize("name,make", [LAYOUTS[0], LAYOUTS[5]], ids=["sod_levels", "cylinder_ib_adapted"])
def test_device_layout_equals_host_with_fused_slopes(name, make):
    p = make()
    topo, state = cases.build(p)
    a, b = _pair(p, topo, state, abi.KG_PREC_MIXED, fuse=True)
    _same_layout(a, b, name + " fused")
    assert len(a.layout_read("r2_list")) > 0
    for g in (a, b):
        g.step(p.dt(), 0, 3)
    _same_state(a, b, name + " fused")
    a.close()
    b.close()


def _cylinder_extra():
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


ADAPT = [
    ("collision_2grids", lambda: cases.collision(center=0.5), lambda: cases.collision(center=0.62)),
    ("cylinder_far_field", lambda: cases.cylinder(scale=0.125, max_level=2, nv=16, vs_levels=0), _cylinder_extra),
]


@pytest.mark.parametrize("name,make_old,make_new", ADAPT, ids=[c[0] for c in ADAPT])
def test_device_layout_after_adaptation(name, make_old, make_new):
    pa, pb = make_old(), make_new()
    ta, sa = cases.build(pa)
    tb, _ = cases.build(pb)
    src = mesh.adapt_sources(ta, tb)
    tb = mesh.adapt_grids(ta, tb, src)
    a, b = _pair(pa, ta, sa, abi.KG_PREC_FP64)
    dt = pa.dt()
    for g in (a, b):
        g.step(dt, 0, 2)
        g.adapt(tb, src)
    _same_layout(a, b, name + " adapted")
    for g in (a, b):
        g.step(dt, 2, 2)
    _same_state(a, b, name + " adapted")
    a.close()
    b.close()


def test_device_layout_equals_host_in_a_batch():
    """Problems admitted to a batch handle: each built on the device and the layouts merged on
    the device equal the host builder's merge, across a release and an admission."""
    from kitgpu.solver import GpuBatch
    probs = [cases.sod(scale=0.125, nv=16), cases.cavity(n=8, nv=12, levels=1, Kn=0.01),
             cases.cylinder(scale=0.125, nv=16, vs_levels=1), cases.collision(center=0.5)]
    built = [cases.build(p) for p in probs]
    prec = abi.KG_PREC_MIXED
    handles = [GpuBatch(abi.make_params(probs[0], precision=prec), 512 << 20, device_flatten=dev) for dev in (True, False)]
    slots = [[], []]
    for b, sl in zip(handles, slots):
        for p, (t, s) in zip(probs[:3], built[:3]):
            sl.append(b.admit(abi.make_params(p, precision=prec, st_check_interval=2), t, s["f"], s["w"], s["prim"], p.dt()))
    _same_layout(handles[0], handles[1], "batch of three")
    for b in handles:
        b.step(2)
    for b, sl in zip(handles, slots):
        b.release(sl[0])
        p3, (t3, s3) = probs[3], built[3]
        b.admit(abi.make_params(p3, precision=prec, st_check_interval=2), t3, s3["f"], s3["w"], s3["prim"], p3.dt())
    _same_layout(handles[0], handles[1], "batch after a release and an admission")
    for b in handles:
        b.step(2)
    for k in slots[0][1:]:
        x, y = handles[0].download(k), handles[1].download(k)
        for key in ("f", "w", "prim", "qf"):
            assert np.array_equal(x[key], y[key]), key
    for b in handles:
        b.close()
