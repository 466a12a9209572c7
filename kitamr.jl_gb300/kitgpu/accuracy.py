"""L-infinity relative errors of the moments between two states of one topology: the
accuracy statement of the mixed form (against the FP64 form or the oracle) and the bar of
the parity tests.  Only fluid cells (bound_enc >= 0) are compared.

Each component is compared against its own largest magnitude over the problem, floored for
components that can be ~0 everywhere:
* ρ, E and T = 1/λ: no floor;
* ρU and U: ρ v_th and v_th (v_th = max sqrt(1/λ), the thermal speed scale);
* q: 5 % of ρ v_th^3 (the free-molecular heat-flux scale; q of a near-equilibrium or
  symmetric flow is close to 0, and FP32 storage of f alone limits q to ~1e-7 ρ v_th^3).
"""
from __future__ import annotations

from typing import Dict

import numpy as np

from . import mesh


def rel_err(a: np.ndarray, b: np.ndarray, floor: float) -> float:
    scale = max(float(np.max(np.abs(b))), floor)
    return float(np.max(np.abs(a - b))) / scale


def moment_errors(topo, ref_w, ref_prim, ref_qf, w, prim, qf) -> Dict[str, float]:
    """Per component: rho, E, T, m<d> (ρU_d), U<d>, q<d>."""
    dim = topo["dim"]
    nw = dim + 2
    be = np.asarray(topo["cell_bound_enc"])
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
        out[f"q{d}"] = rel_err(gq[:, d], rq[:, d], 0.05 * rho * vt ** 3)
    return out


def f_error(topo, ref_f, f) -> float:
    """L-infinity relative error of f over the fluid cells' blocks."""
    be = np.asarray(topo["cell_bound_enc"])
    off = mesh.f_offsets(topo)
    nv_blk = np.diff(off)
    mask = np.repeat(be >= 0, nv_blk)
    return rel_err(f[mask], ref_f[mask], 0.0)


def summary(errs: Dict[str, float]) -> Dict[str, float]:
    """The four quantities of the accuracy statement: ρ, U (largest component), T, q (largest
    component), plus f when present."""
    out = {"rho": errs["rho"], "T": errs["T"],
           "U": max(v for k, v in errs.items() if k.startswith("U")),
           "q": max(v for k, v in errs.items() if k.startswith("q"))}
    if "f" in errs:
        out["f"] = errs["f"]
    return out
