"""Checkpoint payload from the device (kg_download_restart / kg_upload_restart): the state
arrays of save_for_restart (IO/Restart.jl:81-117) against a restatement of its loops, and a
resume through them against an uninterrupted run."""
import numpy as np
import pytest

from kitgpu import abi, cases, mesh

pytestmark = pytest.mark.gpu


def restart_arrays(topo, f, w):
    """save_for_restart's first and second pass over the cells (IO/Restart.jl:87-117): vs_df
    stacks every cell's df (nv x ndf) in cell order, ws holds w per quadrant (zero rows for
    quadrants without a distribution function)."""
    dim, ndf, nc = int(topo["dim"]), int(topo["ndf"]), int(topo["n_cells"])
    nq = int(topo["n_quads"])
    off = mesh.f_offsets(topo)
    nv_total = int(off[nc]) // ndf
    vs_df = np.empty((nv_total, ndf))
    ws = np.zeros((nq, dim + 2))
    row = 0
    w = w.reshape(nc, dim + 2)
    for c in range(nc):
        nv = (int(off[c + 1]) - int(off[c])) // ndf
        df = f[off[c]:off[c + 1]].reshape(ndf, nv).T          # VsData.df (nv x ndf)
        vs_df[row:row + nv, :] = df
        row += nv
        ws[topo["cell_quad"][c], :] = w[c]
    return vs_df, ws


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED], ids=["fp64", "mixed"])
def test_restart_arrays_match_the_reference_layout(prec):
    from kitgpu.solver import GpuStep
    p = cases.cylinder(scale=0.125, max_level=2, nv=16, vs_levels=1)
    topo, state = cases.build(p)
    assert topo["n_quads"] > topo["n_cells"], "the mesh has InsideSolidData quadrants"
    g = GpuStep(abi.make_params(p, precision=prec), topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    g.step(p.dt(), 0, 3)
    st = g.download_state()
    vs_df, ws = g.download_restart(topo["cell_quad"], topo["n_quads"])
    g.close()
    exp_df, exp_ws = restart_arrays(topo, st["f"], st["w"])
    assert np.array_equal(vs_df, exp_df)
    assert np.array_equal(ws, exp_ws)


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED], ids=["fp64", "mixed"])
def test_resume_from_the_checkpoint_is_bit_for_bit(prec):
    """cavity with refinement (no immersed boundary: restart re-initialises the SolidNeighbor
    distributions from their donors, so a run with walls resumes from a different wall state,
    as the reference's restart does): 3 steps, checkpoint, a new handle, 3 more steps == 6."""
    from kitgpu.solver import GpuStep
    p = cases.cavity(n=12, nv=16, levels=1)
    topo, state = cases.build(p)
    prm = abi.make_params(p, precision=prec, st_check_interval=1)
    dt = p.dt()
    a = GpuStep(prm, topo)
    a.upload_state(state["f"], state["w"], state["prim"])
    a.step(dt, 0, 3)
    vs_df, ws = a.download_restart()
    a.step(dt, 3, 3)
    exp = a.download_state()
    a.close()
    b = GpuStep(prm, topo)
    b.upload_restart(vs_df, ws)
    b.step(dt, 3, 3)
    got = b.download_state()
    b.close()
    for k in ("f", "w", "prim", "qf"):
        assert np.array_equal(got[k], exp[k]), k


def test_restart_rejects_bad_quadrant_maps():
    from kitgpu.solver import GpuStep, KitGpuError
    p = cases.cavity(n=8, nv=12)
    topo, state = cases.build(p)
    g = GpuStep(abi.make_params(p), topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    nc = int(topo["n_cells"])
    with pytest.raises(KitGpuError) as e:
        g.download_restart(np.zeros(nc, np.int32), nc)          # repeated rows
    assert e.value.code == 1
    with pytest.raises(KitGpuError):
        g.download_restart(None, nc + 1)                         # n_quads without a map
    g.close()


def test_batch_checkpoint_payload_equals_the_single_handle():
    from kitgpu.solver import GpuBatch, GpuStep
    p = cases.cylinder(scale=0.125, max_level=2, nv=16, vs_levels=1)
    topo, state = cases.build(p)
    q = cases.cavity(n=8, nv=12)
    tq, sq = cases.build(q)
    prm = abi.make_params(p, precision=abi.KG_PREC_MIXED)
    g = GpuStep(prm, topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    g.step(p.dt(), 0, 2)
    exp_df, exp_ws = g.download_restart(topo["cell_quad"], topo["n_quads"])
    g.close()
    b = GpuBatch(prm, pool_bytes=256 << 20)
    s0 = b.admit(abi.make_params(q, precision=abi.KG_PREC_MIXED), tq, sq["f"], sq["w"], sq["prim"], q.dt())
    s1 = b.admit(prm, topo, state["f"], state["w"], state["prim"], p.dt())
    b.step(2)
    vs_df, ws = b.download_restart(s1, topo["cell_quad"], topo["n_quads"])
    b.close()
    assert s0 != s1
    assert np.array_equal(vs_df, exp_df) and np.array_equal(ws, exp_ws)
