"""Serving: a continuous-batching request loop for steady-state solves on one GPU.

Requests (a generated problem each) arrive on a Poisson schedule.  The loop admits every
waiting request whose HBM footprint fits the batch pool (``kg_batch_admit`` refuses with
KG_ERR_BUDGET otherwise and the request waits), advances all admitted problems together
``chunk`` steps at a time with their state resident on the device, and retires a problem
as soon as its density residual -- residual_comm!'s ``sqrt(sumRes * N) / (sumAvg + EPS)``
(src/Solver/Finalize.jl:12-24) -- drops below the tolerance, freeing its slot for the next
arrival.  Latency is arrival to convergence; the loop reports p50 / p99 and solves/s.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional

import numpy as np

from . import abi, cases
from .solver import GpuBatch, KitGpuError

EPS = 1e-12


@dataclass
class Request:
    rid: int
    problem: cases.Problem
    arrival: float                      # seconds after the loop starts
    topo: Optional[Dict] = None
    state: Optional[Dict] = None
    slot: int = -1
    admitted: float = -1.0
    finished: float = -1.0
    steps: int = 0
    residual: float = math.inf
    converged: bool = False
    result: Optional[Dict] = None
    Ma: float = 0.0


def residual_of(rep: abi.KgStepReport, n_quads: int, nw: int) -> np.ndarray:
    sr = np.array(rep.sum_res[:nw])
    sa = np.array(rep.sum_avg[:nw])
    return np.sqrt(sr * n_quads) / (sa + EPS)


def random_request(rng: np.random.Generator, rid: int, arrival: float, small: bool = False) -> Request:
    """A cylinder or cavity steady solve with Ma ~ U[0.1, 5], Kn ~ 10^U(-3, 0), base mesh
    n^2 with n in [32, 96] and velocity grids m^2 with m even in [16, 48] (``small`` shrinks
    the ranges for tests)."""
    kind = rng.choice(["cavity", "cylinder"])
    Kn = float(10 ** rng.uniform(-3, 0))
    if small:
        n = int(rng.integers(6, 12))
        m = int(rng.integers(6, 9)) * 2
    else:
        n = int(rng.integers(32, 97))
        m = int(rng.integers(8, 25)) * 2
    Ma = float(rng.uniform(0.1, 5.0))
    U = Ma * math.sqrt(5.0 / 6.0)
    # velocity domain [-L, L]^2 covering the bulk speed plus five thermal speeds; with an
    # even m, v = 0 stays on a root corner (check_vs_setting)
    L = float(math.ceil(U + 5.0))
    if kind == "cavity":
        p = cases.cavity(n=n, nv=m, levels=0, Kn=Kn, lid=U)
        p.case.quadrature = [-L, L, -L, L]
    else:
        p = cases.cylinder(scale=n / 64.0, max_level=1 if small else 2, nv=m, vs_levels=0, Ma=Ma, Kn=Kn)
        p.case.quadrature = [-L, L, -L, L]
    return Request(rid, p, arrival, Ma=Ma)


@dataclass
class ServeStats:
    latencies: List[float]          # every finished request, arrival to retirement
    solves: int                     # requests that converged
    wall: float
    steps_total: int
    phase_updates: int
    refused: int
    converged_latencies: List[float] = field(default_factory=list)
    steps_to_converge: List[int] = field(default_factory=list)
    unconverged_detail: List[Dict] = field(default_factory=list)

    def summary(self) -> Dict:
        def pct(v, q):
            return float(np.percentile(np.array(v), q) * 1e3) if v else None
        return {"p50_ms": pct(self.latencies, 50), "p99_ms": pct(self.latencies, 99),
                # time to converged steady state, over the requests that converged
                "p50_converged_ms": pct(self.converged_latencies, 50),
                "p99_converged_ms": pct(self.converged_latencies, 99),
                "requests": len(self.latencies), "unconverged": len(self.latencies) - self.solves,
                "solves": self.solves, "solves_per_s": self.solves / self.wall if self.wall > 0 else 0.0,
                "steps_to_converge_max": max(self.steps_to_converge) if self.steps_to_converge else None,
                "wall_s": self.wall, "phase_cell_updates_per_s": self.phase_updates / self.wall if self.wall else 0.0,
                "admissions_refused": self.refused, "unconverged_requests": self.unconverged_detail}


class Server:
    def __init__(self, precision: int = abi.KG_PREC_MIXED, pool_bytes: int = 8 << 30, chunk: int = 20,
                 tol: float = 1e-6, max_steps: int = 20000, device: int = 0, graph: bool = True):
        self.precision = precision
        self.chunk = chunk
        self.tol = tol
        self.max_steps = max_steps
        base = abi.KgParams(dim=2, ndf=2, flux=abi.KG_FLUX_CAIDVM, marching=abi.KG_MARCH_CAIDVM,
                            precision=precision, st_check_interval=chunk)
        self.batch = GpuBatch(base, pool_bytes, device)
        if graph:
            self.batch.use_graph(True)
        self.live: Dict[int, Request] = {}

    def close(self):
        self.batch.close()

    def _admit(self, r: Request, now: float) -> bool:
        if r.topo is None:
            r.topo, r.state = cases.build(r.problem)
        prm = abi.make_params(r.problem, precision=self.precision, st_check_interval=self.chunk)
        try:
            r.slot = self.batch.admit(prm, r.topo, r.state["f"], r.state["w"], r.state["prim"], r.problem.dt(), 0)
        except KitGpuError as e:
            if e.code == 8:
                return False
            raise
        r.admitted = now
        self.live[r.slot] = r
        return True

    def run(self, requests: List[Request], keep_results: bool = False,
            clock: Callable[[], float] = time.perf_counter) -> ServeStats:
        pending = sorted(requests, key=lambda r: r.arrival)
        waiting: List[Request] = []
        done: List[Request] = []
        refused = 0
        t0 = clock()
        steps_total = 0
        updates = 0
        while pending or waiting or self.live:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                waiting.append(pending.pop(0))
            # admit in arrival order while the pool has room
            still = []
            for r in waiting:
                if self._admit(r, now):
                    continue
                refused += 1
                still.append(r)
            waiting = still
            if not self.live:
                if pending:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - (clock() - t0))))
                continue
            reps = self.batch.step(self.chunk)
            steps_total += self.chunk
            now = clock() - t0
            for slot, r in list(self.live.items()):
                r.steps += self.chunk
                updates += self.chunk * int(reps[slot].phase_cells)
                rep = reps[slot]
                if rep.checked:
                    res = residual_of(rep, int(r.topo["n_cells"]), int(r.topo["dim"]) + 2)
                    r.residual = float(res[0])
                if r.residual < self.tol or r.steps >= self.max_steps:
                    r.converged = r.residual < self.tol
                    r.finished = now
                    if keep_results:
                        r.result = self.batch.download(slot)
                    self.batch.release(slot)
                    del self.live[slot]
                    done.append(r)
        wall = clock() - t0
        lat = [r.finished - r.arrival for r in done]
        conv = [r for r in done if r.converged]
        unconv = [dict(kind=r.problem.name, Ma=r.Ma, Kn=r.problem.gas.Kn, cells=int(r.topo["n_cells"]),
                       steps=r.steps, residual=r.residual) for r in done if not r.converged]
        return ServeStats(lat, len(conv), wall, steps_total, updates, refused,
                          [r.finished - r.arrival for r in conv], [r.steps for r in conv], unconv)


def poisson_arrivals(rng: np.random.Generator, rate: float, n: int) -> List[float]:
    gaps = rng.exponential(1.0 / rate, size=n)
    return list(np.cumsum(gaps) - gaps[0])
