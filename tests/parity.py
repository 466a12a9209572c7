"""Shared parity helpers: run a case on the oracle and through libkitgpu.so and compare."""
from __future__ import annotations

import numpy as np

from kitgpu import abi, cases, mesh

# FP64 plain form: 1e-12 relative, per moment component, against the component's
# magnitude over the problem (a component that is ~0 everywhere, e.g. ρV in a 1D tube,
# is compared against ρ's magnitude instead).
TOL_FP64 = 1e-12
# mixed form (FP32 f): 1e-5 relative on ρ, U, T and q
TOL_MIXED = 1e-5


def rel_err(a: np.ndarray, b: np.ndarray, floor: float) -> float:
    scale = max(float(np.max(np.abs(b))), floor)
    return float(np.max(np.abs(a - b))) / scale


def moment_errors(topo, ref_w, ref_prim, ref_qf, w, prim, qf):
    dim = topo["dim"]
    nw = dim + 2
    be = topo["cell_bound_enc"]
    m = be >= 0
    rw, gw = ref_w.reshape(-1, nw)[m], w.reshape(-1, nw)[m]
    rp, gp = ref_prim.reshape(-1, nw)[m], prim.reshape(-1, nw)[m]
    rq, gq = ref_qf.reshape(-1, dim)[m], qf.reshape(-1, dim)[m]
    rho = float(np.max(np.abs(rw[:, 0])))
    vt = float(np.max(np.sqrt(1.0 / rp[:, -1])))
    out = {"rho": rel_err(gw[:, 0], rw[:, 0], 0.0),
           "E": rel_err(gw[:, -1], rw[:, -1], 0.0),
           "T": rel_err(1.0 / gp[:, -1], 1.0 / rp[:, -1], 0.0)}
    for d in range(dim):
        out[f"m{d}"] = rel_err(gw[:, 1 + d], rw[:, 1 + d], rho * vt)
        out[f"U{d}"] = rel_err(gp[:, 1 + d], rp[:, 1 + d], vt)
        # q: relative to its largest magnitude, floored at 10 % of the free-molecular heat-flux
        # scale p v_th = ρ v_th^3 / 2 (q of a near-equilibrium or symmetric flow is close to 0,
        # and FP32 storage of f alone limits q to ~1e-7 ρ v_th^3 absolute)
        out[f"q{d}"] = rel_err(gq[:, d], rq[:, d], 0.05 * rho * vt ** 3)
    return out


def f_error(topo, ref_f, f):
    be = topo["cell_bound_enc"]
    off = mesh.f_offsets(topo)
    mask = np.zeros(ref_f.size, bool)
    for c in np.nonzero(be >= 0)[0]:
        mask[off[c]:off[c + 1]] = True
    return rel_err(f[mask], ref_f[mask], 0.0)


def run_pair(problem, nsteps, precision=abi.KG_PREC_FP64, flux=abi.KG_FLUX_CAIDVM,
             march=abi.KG_MARCH_CAIDVM, chunks=1, check=1, graph=False):
    import oracle as O
    from kitgpu.solver import GpuStep
    topo, state = cases.build(problem)
    prm64 = abi.make_params(problem, precision=abi.KG_PREC_FP64, flux=flux, marching=march, st_check_interval=check)
    prm = abi.make_params(problem, precision=precision, flux=flux, marching=march, st_check_interval=check)
    dt = problem.dt()
    ref = O.OracleState(topo, state).run(prm64, dt, 0, nsteps, nthreads=4)
    g = GpuStep(prm, topo)
    if graph:
        g.use_graph(True)
    g.upload_state(state["f"], state["w"], state["prim"])
    per = nsteps // chunks
    done = 0
    rep = None
    while done < nsteps:
        n = min(per, nsteps - done)
        rep = g.step(dt, done, n)
        done += n
    out = g.download_state()
    out["sw"] = g.download_sw()
    g.close()
    return topo, ref, out, rep
