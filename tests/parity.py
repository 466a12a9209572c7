"""Shared parity helpers: run a case on the oracle and through libkitgpu.so and compare."""
from __future__ import annotations

import os

import numpy as np

from kitgpu import abi, cases
from kitgpu.accuracy import f_error, moment_errors, rel_err  # noqa: F401

# FP64 plain form: 1e-12 relative, per moment component, against the component's
# magnitude over the problem (a component that is ~0 everywhere, e.g. ρV in a 1D tube,
# is compared against ρ's magnitude instead).
TOL_FP64 = 1e-12
# mixed form (FP32 f): 1e-5 relative on ρ, U, T and q
TOL_MIXED = 1e-5
# the oracle's OpenMP threads (all host cores)
ORACLE_THREADS = max(1, os.cpu_count() or 1)


def run_pair(problem, nsteps, precision=abi.KG_PREC_FP64, flux=abi.KG_FLUX_CAIDVM,
             march=abi.KG_MARCH_CAIDVM, chunks=1, check=1, graph=False):
    import oracle as O
    from kitgpu.solver import GpuStep
    topo, state = cases.build(problem)
    prm64 = abi.make_params(problem, precision=abi.KG_PREC_FP64, flux=flux, marching=march, st_check_interval=check)
    prm = abi.make_params(problem, precision=precision, flux=flux, marching=march, st_check_interval=check)
    dt = problem.dt()
    ref = O.OracleState(topo, state).run(prm64, dt, 0, nsteps, nthreads=ORACLE_THREADS)
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
