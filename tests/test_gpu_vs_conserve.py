"""kg_vs_conserve: vs_conserved_correction!'s I-projection of flagged cells on the device against
the oracle's restatement of conserved_I_porjection! (Theory/I-projection.jl:55-158), cell by
cell.  FP64 parity is held at 1e-6 relative: the reference's Newton solve ends on a
rounding-level Armijo decision (see test_gpu_cip.py), so two summation orders may stop one
step apart; the projected moments themselves match w to 1e-7."""
import numpy as np
import pytest

import oracle as O
from kitgpu import abi, cases, mesh

pytestmark = pytest.mark.gpu


def _grid(topo, g):
    dim = topo["dim"]
    go = topo["grid_off"]
    nv = int(go[g + 1] - go[g])
    mid = topo["vs_midpoint"][go[g] * dim:go[g + 1] * dim].reshape(dim, nv).T
    return mid, topo["vs_weight"][go[g]:go[g + 1]]


def _moments(mid, wt, df):
    psi = np.concatenate([np.ones((mid.shape[0], 1)), mid, 0.5 * np.sum(mid ** 2, 1, keepdims=True)], 1)
    w = psi.T @ (wt * df[:, 0])
    if df.shape[1] == 2:
        w[-1] += 0.5 * np.sum(wt * df[:, 1])
    return w


@pytest.mark.parametrize("prec", [abi.KG_PREC_FP64, abi.KG_PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name,make", [
    ("sod_levels", lambda: cases.sod(scale=0.125, nv=16)),
    ("collision_two_grids", lambda: cases.collision()),
    ("box3d", lambda: cases.box3d(n=(6, 4, 4), nv=8, levels=1)),
    ("cylinder_ib", lambda: cases.cylinder(scale=0.25, nv=16, vs_levels=1)),
])
def test_vs_conserve_matches_oracle(name, make, prec):
    from kitgpu.solver import GpuStep
    p = make()
    topo, state = cases.build(p)
    dim, ndf, nc = topo["dim"], topo["ndf"], topo["n_cells"]
    nw = dim + 2
    w = state["w"].reshape(-1, nw).copy()
    w[:, 0] *= 1.01          # targets off the distributions' own moments
    w[:, 1] += 0.01 * w[:, 0]
    w[:, -1] *= 1.02
    flags = np.zeros(nc, np.uint8)
    flags[::2] = 1
    g = GpuStep(abi.make_params(p, precision=prec), topo)
    g.upload_state(state["f"], w.ravel(), state["prim"])
    g.vs_conserve(flags)
    out = g.download_state()
    g.close()
    off = mesh.f_offsets(topo)
    be = topo["cell_bound_enc"]
    f0 = state["f"] if prec == abi.KG_PREC_FP64 else state["f"].astype(np.float32).astype(np.float64)
    worst, mworst, n = 0.0, 0.0, 0
    for c in range(nc):
        blk = slice(off[c], off[c + 1])
        if not flags[c] or be[c] < 0:
            assert np.array_equal(out["f"][blk], f0[blk]), c   # untouched
            continue
        mid, wt = _grid(topo, int(topo["cell_grid"][c]))
        nv = wt.size
        ref, _ = O.iprojection(dim, ndf, mid, wt, state["f"][blk].reshape(ndf, nv).T, w[c])
        got = out["f"][blk].reshape(ndf, nv).T
        worst = max(worst, float(np.max(np.abs(got - ref)) / np.max(np.abs(ref))))
        mworst = max(mworst, float(np.max(np.abs(_moments(mid, wt, got) - w[c])) / np.linalg.norm(w[c])))
        n += 1
    assert n > 0
    print(name, prec, f"f {worst:.1e} moments {mworst:.1e} cells {n}")
    if prec == abi.KG_PREC_FP64:
        assert worst <= 1e-6 and mworst <= 1e-7
    else:
        assert worst <= 1e-5 and mworst <= 1e-5
