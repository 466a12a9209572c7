"""Benchmark of the phase-space step (slope -> flux incl. IB wall -> Shakhov collision).

Headline workload: the 2D Ma 5 / Kn 0.1 cylinder (diffuse isothermal wall, [-8,8]^2, 64x64
trees, 3 levels near the wall, 48^2 velocity roots on [-15,15]^2 adapted by 2 levels), seeded
synthetic initial state; 61 M phase cells, so f is far larger than L2 between steps.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--no-sub]
  python bench.py --mode sphere | sod | batched | serve | adapt | vsadapt   (one workload per line)

Metric: phase-cell updates/s of the mixed-precision form (FP32 f, compensated moments,
FP64 conserved update), with the plain FP64 form, the accuracy of the mixed form against the
FP64 form and of both against the FP64 oracle, the roofline of the dominant kernel, the
oracle CPU baseline and the end-to-end rate through the C-ABI with host buffers beside it.
The default line also carries one compact record per other workload (`sub`): the Sod tube,
the sphere at its benchmark size, the batched form (autotuned) and serving.
N > 1: independent replicas, one per GPU (the path has no exchange on one device).
Other modes:
* sphere: the 3D Ma 3 sphere (``--scale``: base mesh scale of the generator's default
  refinement; without it, the benchmark configuration of about 2.1e5 cells).
* sod: the 2D Sod tube of the reference's Riemann example (inputs inside L2).
* batched: 256 Sod / cavity problems in one batch handle.
* serve: Poisson arrivals solved to residual < 1e-6.
* adapt: one physical-space adaptation of the cylinder on the device (criterion, then the
  refine / coarsen moves of f) against the host route (f down, new topology and f up).
* vsadapt: one velocity-space adaptation of the cylinder on the device.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "kitamr.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

WORKLOAD = "cylinder_ma5_kn0.1_64x64_L3_v48x48_vsL2"
METRIC = "phase-cell updates/s"
UNIT = "updates/s"
# single-problem workloads: name, default scale, generator note
SINGLE = {
    "cylinder": (WORKLOAD, 1.0, "seeded cylinder_buffer_IC state on a generated forest"),
    # the 3D sphere (Ma 3, Kn 0.05, 32^3 trees, 2 levels, 24^3 velocity grid) at its benchmark
    # size: refinement within 3.5 / 1.8 of the wall, about 2.1e5 cells and 2.9e9 phase cells
    # (scale None); a --scale gives the generator's default refinement on a scaled base mesh
    "sphere": ("sphere_ma3_kn0.05_32x32x32_L2_v24x24x24", None, "seeded sphere buffer state on a generated octree"),
    # the 2D Shakhov Sod tube ([0,1]x[0,0.1], 128x4 trees, 2 levels at the jump, 28^2 velocity
    # grid): small enough that f stays in L2 between kernels
    "sod": ("sod_2d_128x4_L2_v28x28", 1.0, "Sod left/right states on a generated forest"),
}


def make_problem(scale=1.0, mode="cylinder"):
    from kitgpu import cases
    if mode == "sphere":
        return cases.sphere_config() if scale is None else cases.sphere(scale=scale)
    if mode == "sod":
        return cases.sod(scale=scale)
    return cases.cylinder(scale=scale, nv=48, vs_levels=2)


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_launch(kernel):
    """dram bytes per launch of `kernel` on the full cylinder, from the committed ncu summary
    (profiles/<kernel>_cylinder.txt), or None."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_cylinder.txt")
    if not os.path.exists(p):
        return None
    m = re.search(r"traffic_bytes_per_full_launch:\s*([0-9.eE+]+)", open(p).read())
    return float(m.group(1)) if m else None


def aggregate(units_local: int, ms_local: float, steps: int, dist=None):
    """Whole-job rate of independent replicas: the units all ranks processed divided by the
    slowest rank's time (max over ranks)."""
    import torch
    ms = float(ms_local)
    units = float(units_local)
    if dist is not None:
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        u = torch.tensor([units], dtype=torch.float64)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        units = float(u.item())
    return units * steps / (ms / 1e3), ms


def pinned_empty(n, torch):
    return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()


def run_single(args, mode, scale, rank, world, dist, e2e=True, march="caidvm"):
    """Timed steps of one single-problem workload in both forms (mixed, then FP64), each on
    a fresh handle, the timed call replaying a CUDA graph; for the mixed form also the
    per-kernel times (a separate pass) and, with e2e, the end-to-end rate through kg_serve.
    Returns (phase cells, per-form results, launches in the timed call, problem, topo, state)."""
    import torch
    from kitgpu import abi, mesh
    from kitgpu.solver import GpuStep

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    from kitgpu import cases
    prob = make_problem(scale, mode)
    topo, state = cases.build(prob)
    P = mesh.phase_cells(topo)
    dt = prob.dt()
    res = {"ndf": int(topo["ndf"])}
    launches_total = 0

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for form, prec in (("mixed", abi.KG_PREC_MIXED), ("fp64", abi.KG_PREC_FP64)):
        mcode = {"caidvm": abi.KG_MARCH_CAIDVM, "cip": abi.KG_MARCH_CIP}[march]
        prm = abi.make_params(prob, precision=prec, st_check_interval=100, marching=mcode)
        g = GpuStep(prm, topo, device=dev)
        g.fuse_slopes(getattr(args, "fuse", "off") == "on")
        g.upload_state(state["f"], state["w"], state["prim"])
        # the timed call replays a CUDA graph of `steps` steps (captured by the last warm-up
        # call, outside the timed region): the same kernels, without per-launch host overhead
        g.use_graph(True)
        step = 0
        for _ in range(args.warmup):
            g.step(dt, step, 1)
            step += 1
        g.step(dt, step, args.steps)
        step += args.steps
        if args.steps % 2:
            # the graph was captured at the parity of the f buffers before the call: bring it back
            g.step(dt, step, 1)
            step += 1
        sampler = ClockSampler(dev) if form == "mixed" else None
        barrier()
        if sampler:
            sampler.start()
            time.sleep(0.3)
        rep = g.step(dt, step, args.steps)
        barrier()
        clocks = sampler.stop() if sampler else None
        step += args.steps
        value, ms = aggregate(P, rep.device_ms, args.steps, dist)
        res[form] = dict(ms_per_step=ms / args.steps, value=value, launches=rep.kernel_launches)
        if form == "mixed":
            launches_total = rep.kernel_launches
            res[form]["clocks"] = clocks
            # per-kernel device times (CUDA events on the handle's stream), separate pass
            g.profile(True)
            g.step(dt, step, 3)
            step += 3
            res[form]["kernels"] = g.profile_read()
            g.profile(False)
        if form == "mixed" and e2e:
            # end to end through the C-ABI with pinned host buffers: kg_serve runs one request
            # of one step per timed step; every request uploads f, w, prim from the host and
            # downloads f, w, prim, qf (the upload of the next and the download of the previous
            # request overlap the step, both link directions at once)
            ins = {"f": pinned_empty(state["f"].size, torch), "w": pinned_empty(state["w"].size, torch),
                   "prim": pinned_empty(state["prim"].size, torch)}
            for k in ins:
                ins[k][:] = state[k]
            outs = [{"f": pinned_empty(state["f"].size, torch), "w": pinned_empty(state["w"].size, torch),
                     "prim": pinned_empty(state["prim"].size, torch),
                     "qf": pinned_empty(topo["n_cells"] * topo["dim"], torch)} for _ in range(2)]
            g.use_graph(False)
            e2e_steps = max(1, args.steps)     # one request per timed step
            requests = [ins] * e2e_steps
            req_out = [outs[r % 2] for r in range(e2e_steps)]
            # untimed warm-up requests: the handle's serving staging (three f blocks in FP64) and
            # copy streams are made on first use
            g.serve(requests[:2], dt, step, 1, outputs=req_out[:2])
            barrier()
            t0 = time.perf_counter()
            g.serve(requests, dt, step, 1, outputs=req_out)
            barrier()
            el = time.perf_counter() - t0
            if dist is not None:
                t = torch.tensor([el], dtype=torch.float64)
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                el = float(t.item())
            h2d = sum(a.nbytes for a in ins.values())
            d2h = sum(a.nbytes for a in outs[0].values())
            res[form]["e2e"] = {"value": P * world * e2e_steps / el, "unit": UNIT,
                                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)}
            del ins, outs, requests, req_out
        g.close()
    res["graph"] = True
    return P, res, launches_total, prob, topo, state


def accuracy_single(prob, topo, state, acc_steps, oracle_steps, threads, oracle_f=True, march="caidvm"):
    """The accuracy statement of one workload, from its initial state:
    * mixed_vs_fp64: the mixed form against the FP64 form, both on the GPU, after acc_steps;
    * fp64_vs_oracle / mixed_vs_oracle: each form against the FP64 CPU oracle after
      oracle_steps (0: not run), with f's error too when oracle_f.
    L-infinity relative errors of ρ, U, T and q over the fluid cells (kitgpu.accuracy)."""
    import torch
    from kitgpu import abi
    from kitgpu.accuracy import f_error, moment_errors, summary
    from kitgpu.solver import GpuStep
    dev = torch.cuda.current_device()
    dt = prob.dt()
    mcode = {"caidvm": abi.KG_MARCH_CAIDVM, "cip": abi.KG_MARCH_CIP}[march]
    snaps = {}
    for form, prec in (("fp64", abi.KG_PREC_FP64), ("mixed", abi.KG_PREC_MIXED)):
        g = GpuStep(abi.make_params(prob, precision=prec, st_check_interval=100, marching=mcode), topo, device=dev)
        g.upload_state(state["f"], state["w"], state["prim"])
        done = 0
        if oracle_steps:
            g.step(dt, 0, oracle_steps)
            done = oracle_steps
            snaps[(form, "oracle")] = g.download_state(f=oracle_f)
        if acc_steps > done:
            g.step(dt, done, acc_steps - done)
        snaps[(form, "acc")] = snaps[(form, "oracle")] if acc_steps == done else g.download_state(f=False)
        g.close()
    a, b = snaps[("fp64", "acc")], snaps[("mixed", "acc")]
    out = {"mixed_vs_fp64": dict(summary(moment_errors(topo, a["w"], a["prim"], a["qf"], b["w"], b["prim"], b["qf"])),
                                 steps=acc_steps)}
    if oracle_steps:
        import oracle as O
        prm64 = abi.make_params(prob, precision=abi.KG_PREC_FP64, st_check_interval=100, marching=mcode)
        ref = O.OracleState(topo, state).run(prm64, dt, 0, oracle_steps, nthreads=threads)
        for form in ("fp64", "mixed"):
            g = snaps[(form, "oracle")]
            e = moment_errors(topo, ref.w, ref.prim, ref.qf, g["w"], g["prim"], g["qf"])
            if oracle_f:
                e["f"] = f_error(topo, ref.f, g["f"])
            out[f"{form}_vs_oracle"] = dict(summary(e), steps=oracle_steps)
        del ref
    out["tolerance"] = {"mixed": 1e-5, "fp64_vs_oracle": 1e-12}
    out["mixed_form"] = ("FP32 f / sdf and per-velocity arithmetic (packed FP32x2 in the 2D regular-cell kernel), "
                         "per-thread FP32 moment sums (compensated in the generic kernel) reduced in float-float to "
                         "FP64, FP64 conserved update and primitive recovery; the Maxwellian exponent formed in "
                         "float-float (~44 bits) and tau / Shakhov / relaxation constants in FP32 from the FP64 "
                         "primitives (a departure from an all-FP64 exponent, held to the same 1e-5)")
    return out


FLUX_KERNELS = ("flux_packed_kernel", "flux_packed_kernel_r2", "flux_packed_inner_kernel", "flux_packed_inner_kernel_paired",
                "flux_regular_kernel",
                "flux_collide_kernel")


def roofline_of(kern, P, ndf, peak, peak_kind, traffic=None):
    """Roofline of the dominant flux kernel (the flux kernel with the largest device time) from
    its per-launch CUDA-event time: 2 * NDF * 4 B per phase cell it processed (one read and one
    write of f in FP32) over that time, against the measured HBM peak.  `flux_kernels` gives
    the same per flux kernel, `flux_step` for all flux kernels of a step together (the
    profiling pass launches them one after another)."""
    fk = {k: v for k, v in kern.items() if k in FLUX_KERNELS and v[1] > 0}
    if not fk:
        return None
    if all(len(v) < 3 or v[2] == 0 for v in fk.values()):
        # no per-kernel phase cells: all flux kernels over the problem's phase cells
        ms = sum(v[0] for v in fk.values())
        cnt = max(v[1] for v in fk.values())
        fk = {"flux_collide_kernel": (ms, cnt, P * cnt)}
    name = max(fk, key=lambda k: fk[k][0])
    ms, cnt, units = fk[name][:3]
    avg_s = ms / cnt / 1e3
    b_alg = 2 * ndf * 4 * units / cnt
    ach = b_alg / avg_s / 1e9
    per = {}
    for k, v in fk.items():
        lb = 2 * ndf * 4 * v[2] / v[1]
        per[k] = {"launch_ms": v[0] / v[1], "phase_cells": int(v[2] // v[1]),
                  "achieved": lb / (v[0] / v[1] / 1e3) / 1e9, "frac": lb / (v[0] / v[1] / 1e3) / 1e9 / peak}
    steps = cnt
    step_ms = sum(v[0] for v in fk.values()) / steps
    step_b = 2 * ndf * 4 * sum(v[2] for v in fk.values()) / steps
    return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
            "traffic": traffic, "kernel": name, "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": b_alg, "launch_ms": avg_s * 1e3, "flux_kernels": per,
            "flux_step": {"ms": step_ms, "algorithmic_bytes": step_b,
                          "achieved": step_b / (step_ms / 1e3) / 1e9,
                          "frac": step_b / (step_ms / 1e3) / 1e9 / peak}}


def batch_shapes():
    """Eight mesh / velocity-grid shapes of the batched workload (Sod tubes and lid-driven
    cavities, base meshes 32^2..128^2-class, 0-2 levels, velocity grids 16^2..40^2 on [-6,6]^2)."""
    from kitgpu import cases
    out = []
    for n, lev, m in ((32, 0, 16), (48, 1, 24), (64, 1, 32), (40, 2, 20)):
        p = cases.cavity(n=n, nv=m, levels=lev)
        out.append(("cavity", p, cases.build(p)))
    for sc, lev, m in ((0.25, 2, 24), (0.5, 1, 28), (0.75, 2, 40), (0.5, 0, 16)):
        p = cases.sod(scale=sc, max_level=lev, nv=m)
        p.case.quadrature = [-6.0, 6.0, -6.0, 6.0]
        out.append(("sod", p, cases.build(p)))
    return out


def run_batched(args, autotune=True):
    """Config 4: 256 problems in one batch handle, CUDA-graph replay, the flux schedule chosen
    by kg_autotune (one CTA per cell, or persistent CTAs in natural or largest-first order).
    Accuracy: one problem of each shape, mixed against FP64, after the same steps."""
    import torch
    from kitgpu import abi, mesh
    from kitgpu.accuracy import moment_errors, summary
    from kitgpu.solver import GpuBatch
    shapes = batch_shapes()
    forms = {}
    snaps = {}
    for form, prec in (("mixed", abi.KG_PREC_MIXED), ("fp64", abi.KG_PREC_FP64)):
        rng = np.random.default_rng(20261203 + 4)
        base = abi.make_params(shapes[0][1], precision=prec, st_check_interval=100)
        free = torch.cuda.mem_get_info()[0]
        b = GpuBatch(base, int(free * 0.85))
        b.use_graph(True)
        P = 0
        slots = []
        for k in range(args.problems):
            name, prob, (topo, state) = shapes[k % len(shapes)]
            prob.gas.Kn = float(10 ** rng.uniform(-3, 0))
            prm = abi.make_params(prob, precision=prec, st_check_interval=100)
            slots.append(b.admit(prm, topo, state["f"], state["w"], state["prim"], prob.dt(), 0))
            P += mesh.phase_cells(topo)
        if autotune:
            b.autotune(True)
        for _ in range(args.warmup):
            b.step(1)
        reps = b.step(args.steps)       # graph capture of `steps` steps
        reps = b.step(args.steps)       # replay, timed
        ms = next(iter(reps.values())).device_ms
        forms[form] = {"value": P * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps, "phase_cells": P,
                       "launches_per_call": int(next(iter(reps.values())).kernel_launches)}
        if autotune:
            forms[form]["autotune"] = b.autotune_result()
        for k in range(len(shapes)):
            snaps[(form, k)] = b.download(slots[k])
        if form == "mixed":
            # per-kernel device times (CUDA events on the handle's stream), a separate pass
            b.profile(True)
            b.step(2)
            forms[form]["kernels_ms_per_step"] = {k: v[0] / 2 for k, v in b.profile_read().items()}
            forms[form]["kernels"] = b.profile_read()
            b.profile(False)
        b.close()
    acc = {}
    for k in range(len(shapes)):
        topo = shapes[k][2][0]
        a, m = snaps[("fp64", k)], snaps[("mixed", k)]
        e = summary(moment_errors(topo, a["w"], a["prim"], a["qf"], m["w"], m["prim"], m["qf"]))
        for q, v in e.items():
            acc[q] = max(acc.get(q, 0.0), v)
    acc["steps"] = args.warmup + 2 * args.steps
    acc["problems_compared"] = len(shapes)
    m = forms["mixed"]
    return {"metric": METRIC + " (batched)", "value": m["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-f/f64-moments", "data": "synthetic",
            "config": {"workload": f"batched_{args.problems}_sod_cavity_8_shapes", "phase_cells": m["phase_cells"],
                       "graph": True, "autotune": autotune},
            "forms": forms, "mixed_over_fp64": forms["mixed"]["value"] / forms["fp64"]["value"],
            "accuracy": {"mixed_vs_fp64": acc}, "gpu_launches": m["launches_per_call"]}


def run_serve(args, requests=None, rate=None, forms=None):
    """Config 5: Poisson arrivals of cylinder / cavity steady solves, continuous batching,
    each request to a density residual below 1e-6 (or the step cap, counted as unconverged).
    Latency percentiles over all requests and over the converged ones."""
    import torch
    from kitgpu import abi, cases, serve
    nreq = requests or args.requests
    lam = rate or args.rate
    rng = np.random.default_rng(20261203 + 5)
    arrivals = serve.poisson_arrivals(rng, lam, nreq)
    reqs = [serve.random_request(rng, i, a, small=False) for i, a in enumerate(arrivals)]
    for r in reqs:   # generate before the clock starts
        r.topo, r.state = cases.build(r.problem)
    out = {}
    allforms = (("mixed", abi.KG_PREC_MIXED), ("fp64", abi.KG_PREC_FP64))
    for form, prec in [x for x in allforms if x[0] in (forms or args.forms).split(",")]:
        for r in reqs:
            r.slot, r.admitted, r.finished, r.steps, r.residual, r.converged = -1, -1.0, -1.0, 0, float("inf"), False
        free = torch.cuda.mem_get_info()[0]
        srv = serve.Server(precision=prec, pool_bytes=int(free * 0.8), chunk=50, tol=1e-6, max_steps=args.max_steps)
        st = srv.run(reqs)
        srv.close()
        out[form] = st.summary()
    m = out["mixed"]
    return {"metric": "serve p50/p99 time-to-steady-state", "value": m["p99_ms"], "unit": "ms", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-f/f64-moments", "data": "synthetic",
            "config": {"workload": f"serve_poisson_{lam}_per_s_{nreq}_requests", "tol": 1e-6,
                       "step_cap": args.max_steps, "cfl": 0.4},
            "forms": out}


def cylinder_after_adaptation():
    """The cylinder mesh after one physical-space adaptation: a band refined downstream and
    the outer level-1 ring coarsened upstream; the cells at the wall are unchanged."""
    p = make_problem(1.0)
    base = p.case.refine

    def refine(mid, ds, L):
        if L == 0 and mid[0] > 5.0 and abs(mid[1]) < 2.0:
            return True
        if L == 1 and mid[0] < -3.0:
            return False
        return base(mid, ds, L)
    p.case.refine = refine
    return p


def run_vsadapt(args):
    """Cost of one velocity-space adaptation of the cylinder (mixed form) on the device: the
    flags (kg_vs_flags), the df moves onto refined grids (kg_adapt with KG_ADAPT_VS: the host
    flattening of the new topology plus the device move) and the conservative correction of
    the changed cells (kg_vs_conserve), then the same back onto the original grids.  The new
    grids (every non-donor fluid cell's grid refined where |u| < 1.5) are built before the
    timed region: that is the caller's host work.  Compared with the route that keeps f on
    the host (f down and up around the reference's own host adaptation)."""
    import torch
    from kitgpu import abi, cases, mesh
    from kitgpu.solver import GpuStep
    pa = make_problem(1.0)
    ta, sa = cases.build(pa)
    dim = ta["dim"]
    root = mesh.vgrid_root_ds(pa.case.quadrature, pa.case.vs_trees_num, dim)
    donors = set(int(x) for x in np.asarray(ta["wall_donor"]))
    be = ta["cell_bound_enc"]
    by_grid = {}
    for g in np.unique(ta["cell_grid"]):
        c0 = int(np.nonzero(ta["cell_grid"] == g)[0][0])
        vg = mesh.cell_vgrid(ta, c0)
        ok = (np.linalg.norm(vg.midpoint, axis=1) < 1.5) & (vg.level < pa.vs_maxlevel)
        by_grid[int(g)] = mesh.refine_vgrid(vg, ok, root)
    changed = [c for c in range(ta["n_cells"]) if be[c] >= 0 and c not in donors]
    tb = mesh.with_cell_vgrids(ta, {c: by_grid[int(ta["cell_grid"][c])] for c in changed})
    src_b, src_a = mesh.vs_sources(tb), mesh.vs_sources(ta)
    flags = np.zeros(ta["n_cells"], np.uint8)
    flags[changed] = 1
    prm = abi.make_params(pa, precision=abi.KG_PREC_MIXED, st_check_interval=100)
    cfg = abi.make_vs_config(pa)
    dt = pa.dt()
    g = GpuStep(prm, ta)
    g.upload_state(sa["f"], sa["w"], sa["prim"])
    g.step(dt, 0, args.warmup)
    step = args.warmup
    t_flags, t_move, t_cons = [], [], []
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.vs_flags(cfg, eta=False)
        t1 = time.perf_counter()
        g.adapt(tb, src_b) if k % 2 == 0 else g.adapt(ta, src_a)
        t2 = time.perf_counter()
        g.vs_conserve(flags)
        t3 = time.perf_counter()
        t_flags.append((t1 - t0) * 1e3); t_move.append((t2 - t1) * 1e3); t_cons.append((t3 - t2) * 1e3)
        g.step(dt, step, 1)
        step += 1
    g.close()
    # host route: f (and sdf for the flags' criterion) down, a state of the new size up
    h = GpuStep(prm, ta)
    h.upload_state(sa["f"], sa["w"], sa["prim"])
    h.step(dt, 0, 1)
    host = []
    for k in range(max(3, args.steps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = h.download_state(sdf=True)
        h.upload_state(out["f"], out["w"], out["prim"])
        host.append((time.perf_counter() - t0) * 1e3)
    h.close()
    med = lambda v: float(np.median(v))
    total = med([a + b + c for a, b, c in zip(t_flags, t_move, t_cons)])
    return {"metric": "velocity-space adaptation time (flags + grid moves + conservative correction)",
            "value": total, "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32-f/f64-moments",
            "data": "synthetic",
            "config": {"workload": WORKLOAD + " velocity grids refined where |u| < 1.5 and back",
                       "changed_cells": len(changed), "phase_cells": [mesh.phase_cells(ta), mesh.phase_cells(tb)]},
            "device_route": {"vs_flags_ms": med(t_flags), "adapt_vs_ms": med(t_move), "vs_conserve_ms": med(t_cons)},
            "host_route_transfer_ms": med(host), "gpu_launches": None}


def run_adapt(args):
    """Cost of one physical-space adaptation of the cylinder (mixed form): the device route
    (kg_criterion, then kg_adapt with the new topology and the per-cell sources) against the
    host route it replaces (f down, the new topology and f up)."""
    import torch
    from kitgpu import abi, cases, mesh
    from kitgpu.solver import GpuStep
    pa = make_problem(1.0)
    ta, sa = cases.build(pa)
    tb, _ = cases.build(cylinder_after_adaptation())
    fwd = mesh.adapt_sources(ta, tb)
    tb = mesh.adapt_grids(ta, tb, fwd)
    back = mesh.adapt_sources(tb, ta)
    ta2 = mesh.adapt_grids(tb, ta, back)
    kinds = np.bincount(fwd["kind"], minlength=3)
    prm = abi.make_params(pa, precision=abi.KG_PREC_MIXED, st_check_interval=100)
    dt = pa.dt()
    g = GpuStep(prm, ta)
    g.upload_state(sa["f"], sa["w"], sa["prim"])
    g.step(dt, 0, args.warmup)
    step = args.warmup
    crit, adapt = [], []
    g.profile(True)         # host phase times of kg_adapt (the steps between run untimed)
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.criterion(0.05)
        t1 = time.perf_counter()
        g.adapt(tb, fwd) if k % 2 == 0 else g.adapt(ta2, back)
        t2 = time.perf_counter()
        crit.append((t1 - t0) * 1e3)
        adapt.append((t2 - t1) * 1e3)
        g.step(dt, step, 1)
        step += 1
    phases = {k: v[0] / max(v[1], 1) for k, v in g.profile_read().items() if k.startswith(("adapt:", "rebuild:", "flatten:"))}
    g.close()
    # flattening alone (host), the part of kg_adapt that is not device work
    from kitgpu.solver import load_library
    import ctypes as C
    L = load_library()
    tref = abi.TopologyRef(tb)
    b = C.c_int64()
    t0 = time.perf_counter()
    L.kg_topology_footprint(C.byref(prm), C.cast(tref.ptr, C.c_void_p), C.byref(b))
    flatten_ms = (time.perf_counter() - t0) * 1e3
    # host route: download f / w / prim, upload the new topology and a state of its size
    h = GpuStep(prm, ta)
    h.upload_state(sa["f"], sa["w"], sa["prim"])
    h.step(dt, 0, 1)
    nfb = int(mesh.f_offsets(tb)[-1])
    fb = np.ones(nfb)
    wb = np.tile(sa["w"][:4], tb["n_cells"])
    host = []
    for k in range(max(3, args.steps // 4)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = h.download_state()
        t1 = time.perf_counter()
        if k % 2 == 0:
            L.kg_upload_topology(h.h, C.cast(tref.ptr, C.c_void_p))
            h.L.kg_upload_state(h.h, fb.ctypes.data, wb.ctypes.data, wb.ctypes.data)
            h.nc, h.foff = int(tb["n_cells"]), mesh.f_offsets(tb)
        else:
            ta_ref = abi.TopologyRef(ta)
            L.kg_upload_topology(h.h, C.cast(ta_ref.ptr, C.c_void_p))
            h.L.kg_upload_state(h.h, sa["f"].ctypes.data, sa["w"].ctypes.data, sa["prim"].ctypes.data)
            h.nc, h.foff = int(ta["n_cells"]), mesh.f_offsets(ta)
        t2 = time.perf_counter()
        host.append(((t1 - t0) * 1e3, (t2 - t1) * 1e3, out["f"].nbytes))
    h.close()
    med = lambda v: float(np.median(v))
    dev_total = med([a + b_ for a, b_ in zip(crit, adapt)])
    host_total = med([a + b_ for a, b_, _ in host])
    return {"metric": "physical-space adaptation time (criterion + refine/coarsen of the state)", "value": dev_total,
            "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-f/f64-moments", "data": "synthetic",
            "config": {"workload": WORKLOAD + " adapted: band refined downstream, ring coarsened upstream",
                       "cells": [int(ta["n_cells"]), int(tb["n_cells"])], "kept": int(kinds[0]),
                       "refined": int(kinds[1]), "coarsened": int(kinds[2]),
                       "phase_cells": [mesh.phase_cells(ta), mesh.phase_cells(tb)]},
            "device_route": {"criterion_ms": med(crit), "adapt_ms": med(adapt), "flatten_ms": flatten_ms,
                             "adapt_phases_ms": phases,
                             "lohner_bytes_down": int(ta["n_cells"]) * 8 * 8},
            "host_route": {"download_ms": med([x[0] for x in host]), "upload_ms": med([x[1] for x in host]),
                           "total_ms": host_total, "f_bytes_down": int(host[0][2]),
                           "note": "transfers and re-upload only; the host-side interpolation itself is extra"},
            "device_over_host": dev_total / host_total}


def cpu_baseline(threads, budget_s=12.0, mode="cylinder", scale=1.0, built=None):
    """The FP64 oracle on the host cores (OpenMP, `threads`), on the same workload as the GPU
    line, for about budget_s seconds of steps (at least one)."""
    import oracle as O
    from kitgpu import abi, cases, mesh
    if built is None:
        prob = make_problem(scale=scale, mode=mode)
        topo, state = cases.build(prob)
    else:
        prob, topo, state = built
    P = mesh.phase_cells(topo)
    st = O.OracleState(topo, state)
    prm = abi.make_params(prob, st_check_interval=100)
    n, t0 = 0, time.perf_counter()
    while True:
        st.run(prm, prob.dt(), n, 1, nthreads=threads)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or n >= 40:
            break
    return {"value": P * n / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{mode} workload as measured ({P} phase cells), {n} steps from the initial state, FP64"}


def sub_single(args, mode, threads, acc_steps, oracle_steps, oracle_f=True):
    """A compact record of one single-problem workload: rate of both forms, per-kernel times,
    roofline of the flux kernel and the accuracy statement."""
    import copy
    a = copy.copy(args)
    a.steps, a.warmup = min(args.steps, 10), 3     # a compact record: 10 timed steps per form
    P, res, launches, prob, topo, state = run_single(a, mode, SINGLE[mode][1], 0, 1, None, e2e=False)
    peak, peak_kind = measured_peaks()
    kern = res["mixed"].get("kernels", {})
    rec = {"workload": SINGLE[mode][0], "phase_cells": P, "cells": int(topo["n_cells"]),
           "value": res["mixed"]["value"], "unit": UNIT, "steps": a.steps,
           "ms_per_step": res["mixed"]["ms_per_step"],
           "fp64": {"value": res["fp64"]["value"], "ms_per_step": res["fp64"]["ms_per_step"]},
           "kernels_ms": {k: {"total_ms": v[0], "launches": v[1], "phase_cells": v[2]} for k, v in kern.items()},
           "roofline": roofline_of(kern, P, res["ndf"], peak, peak_kind), "gpu_launches": launches}
    rec["accuracy"] = accuracy_single(prob, topo, state, acc_steps, oracle_steps, threads, oracle_f=oracle_f)
    if oracle_steps == 0:
        rec["accuracy"]["oracle"] = "not run at this size in the default line (the FP64 oracle takes ~40 s per step here)"
    return rec


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sub", action="store_true", help="headline only: no per-workload sub-records")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the accuracy passes")
    ap.add_argument("--scale", type=float, default=None,
                    help="scale of the base mesh (default: the workload's own; smaller for profiling captures)")
    ap.add_argument("--mode", default="cylinder", choices=["cylinder", "sphere", "sod", "batched", "serve", "adapt", "vsadapt"])
    ap.add_argument("--problems", type=int, default=256, help="batched: number of problems")
    ap.add_argument("--rate", type=float, default=50.0, help="serve: Poisson arrival rate (req/s)")
    ap.add_argument("--requests", type=int, default=64, help="serve: number of requests")
    ap.add_argument("--max-steps", type=int, default=20000, help="serve: step cap of a request")
    ap.add_argument("--forms", default="mixed,fp64", help="serve: precision forms to run (mixed, fp64)")
    ap.add_argument("--fuse", default="off", choices=["on", "off"],
                    help="slopes of regular cells in the flux kernel (kg_fuse_slopes; the same results)")
    ap.add_argument("--march", default="caidvm", choices=["caidvm", "cip"],
                    help="single-problem modes: time marching (cip: CIP_Marching, meshes without walls)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.scale is None and args.mode in SINGLE:
        args.scale = SINGLE[args.mode][1]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo")
        dist = dist_mod
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        # The reference is Julia and cannot run on this machine; its CPU path is the oracle port,
        # timed on the headline workload itself (every step a full step of all 61 M phase cells).
        if rank != 0:
            return
        import oracle as O
        from kitgpu import abi, cases, mesh
        prob = make_problem(scale=1.0)
        topo, state = cases.build(prob)
        P = mesh.phase_cells(topo)
        st = O.OracleState(topo, state)
        prm = abi.make_params(prob, st_check_interval=100)
        for s in range(args.warmup):
            st.run(prm, prob.dt(), s, 1, nthreads=threads)
        t0 = time.perf_counter()
        st.run(prm, prob.dt(), args.warmup, args.steps, nthreads=threads)
        el = time.perf_counter() - t0
        v = P * args.steps / el
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded cylinder_buffer_IC state on a generated forest)",
                "config": {"workload": WORKLOAD, "phase_cells": P, "form": "fp64 (CPU oracle)",
                           "parallelism": f"host threads ({threads})"},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": f"the full workload ({P} phase cells per step), {args.steps} timed steps "
                                           f"after {args.warmup}, FP64 oracle; the reference's Julia path is "
                                           "unavailable on this box"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.mode == "batched":
        line = run_batched(args)
        if rank == 0:
            print(json.dumps(line))
        return
    if args.mode == "serve":
        line = run_serve(args)
        if rank == 0:
            print(json.dumps(line))
        return
    if args.mode in ("adapt", "vsadapt"):
        line = run_adapt(args) if args.mode == "adapt" else run_vsadapt(args)
        if rank == 0:
            print(json.dumps(line))
        return
    P, res, launches, prob, topo, state = run_single(args, args.mode, args.scale, rank, world, dist, e2e=True,
                                                     march=args.march)
    if rank != 0:
        return
    wname, wscale, wdata = SINGLE[args.mode]
    ndf = res["ndf"]
    peak, peak_kind = measured_peaks()
    mixed = res["mixed"]
    kern = mixed.get("kernels", {})
    roof = roofline_of(kern, P, ndf, peak, peak_kind)
    if roof and args.mode == "cylinder" and args.scale == 1.0:
        roof["traffic"] = ncu_traffic_per_launch(roof["kernel"])
    line = {
        "metric": METRIC, "value": mixed["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mixed["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-f/f64-moments",
        "data": f"synthetic ({wdata})",
        "config": {"workload": wname if args.scale == wscale else f"{wname} at scale {args.scale}",
                   "phase_cells": P, "form": "mixed",
                   "l2": (f"inputs > L2 (f is {P * ndf * 4 / 1e6:.0f} MB FP32, sdf {P * ndf * 4 * (2 if ndf == 2 else 3) / 1e6:.0f} MB)"
                          if P * ndf * 4 * (3 if ndf == 2 else 4) > 129e6 else
                          f"inputs inside L2 (f {P * ndf * 4 / 1e6:.0f} MB FP32), not flushed between steps: the workload is this small"),
                   "parallelism": f"replicas{world}", "cuda_graph": True, "marching": args.march},
        "forms": {"mixed": {"value": mixed["value"], "ms_per_step": mixed["ms_per_step"]},
                  "fp64": {"value": res["fp64"]["value"], "ms_per_step": res["fp64"]["ms_per_step"]}},
        "kernels_ms": {k: {"total_ms": v[0], "launches": v[1], "phase_cells": v[2]} for k, v in kern.items()},
        "roofline": roof,
        "e2e": mixed.get("e2e"),
        "gpu_launches": launches,
        "clocks": mixed.get("clocks"),
    }
    if not args.no_accuracy and world == 1:
        big = P * ndf > 4e9        # the oracle of a multi-GB-f workload is too slow for this line
        acc_steps = 10 if big else 100
        oracle_steps = 0 if big else (100 if P < 2e6 else 2)
        line["accuracy"] = accuracy_single(prob, topo, state, acc_steps, oracle_steps, threads, march=args.march)
    if not args.no_cpu and world == 1:
        line["cpu_baseline"] = cpu_baseline(threads, mode=args.mode, built=(prob, topo, state))
    del topo, state
    if args.mode == "cylinder" and args.scale == 1.0 and not args.no_sub and world == 1:
        # one compact record per other workload of the benchmark, so that every one of them
        # is measured in the default run
        sub = {}
        t0 = time.perf_counter()
        sub["sod"] = sub_single(args, "sod", threads, acc_steps=100, oracle_steps=100)
        sub["sphere"] = sub_single(args, "sphere", threads, acc_steps=10, oracle_steps=0)
        b = run_batched(args)
        sub["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "config", "mixed_over_fp64",
                                             "accuracy", "gpu_launches")}
        sub["batched"]["fp64"] = {k: b["forms"]["fp64"][k] for k in ("value", "ms_per_step")}
        bk = b["forms"]["mixed"].get("kernels", {})
        sub["batched"]["roofline"] = roofline_of(bk, b["config"]["phase_cells"], 2, peak, peak_kind)
        sub["batched"]["autotune"] = b["forms"]["mixed"].get("autotune")
        # the mixed form only: the FP64 form of the same 12 requests takes ~10 minutes
        # (``--mode serve`` runs both)
        sv = run_serve(args, requests=12, rate=20.0, forms="mixed")
        sub["serve"] = {"config": sv["config"], "forms": sv["forms"]}
        sub["wall_s"] = time.perf_counter() - t0
        line["sub"] = sub
    print(json.dumps(line))


if __name__ == "__main__":
    main()
