"""The synthetic workloads: seeded stand-ins for the reference's examples and for the
configurations the benchmark is quoted on.  Every case is a ``mesh.Case`` plus the gas
and solver parameters; ``scale`` shrinks a case for CPU-sized parity tests.

* ``sod``       2D Shakhov Sod tube (example/Riemann_problem/rp_1D.jl), [0,1]x[0,0.1],
                128x4 trees, 2 refinement levels around the interface, 28^2 velocity
                grid on [-5,5]^2, outflow in x, periodic in y.
* ``couette``   the reference's own test (test/runtests.jl): 16x16 box, Maxwellian walls in
                x (one moving at sqrt(5/6)), periodic in y, 16^2 velocity grid.
* ``cavity``    lid-driven cavity, four Maxwellian walls, lid speed 0.15.
* ``cylinder``  Ma 5, Kn 0.1 flow past a diffuse isothermal cylinder of radius 1,
                [-8,8]^2, 64x64 trees, 3 levels near the wall, 48^2 velocity roots on
                [-15,15]^2 adapted by up to 2 levels around the local bulk velocity.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Dict, Optional, Tuple

import numpy as np

from . import mesh as M


@dataclass
class Gas:
    Kn: float = 0.05
    Pr: float = 2.0 / 3.0
    K: float = 1.0
    gamma: float = 5.0 / 3.0
    omega: float = 0.81
    alpha_r: float = 1.0
    omega_r: float = 0.81

    def mu_ref(self) -> float:
        # ref_vhs_vis(Kn, omega, alpha) called as ref_vhs_vis(Kn, αᵣ, ωᵣ) (Gas/Types.jl:33):
        # the reference passes αᵣ as `omega` and ωᵣ as `alpha`; reproduced as written.
        omega_arg, alpha_arg = self.alpha_r, self.omega_r
        mu0 = (5.0 * (alpha_arg + 1.0) * (alpha_arg + 2.0) * math.sqrt(math.pi)
               / (4.0 * alpha_arg * (5.0 - 2.0 * omega_arg) * (7.0 - 2.0 * omega_arg)) * self.Kn)
        return mu0 * 1.0 ** (0.5 - omega_arg)


# The reference's default CFL (src/Solver/Types.jl:122) and the one of its examples
# (example/Riemann_problem/rp_1D.jl:14, rp_2D.jl:29, blast_wave/bw_2D.jl:34).  Its wall
# treatment (one-sided unlimited slope, plain reconstruction at a Maxwellian wall) is not
# stable at CFL 0.8: a lid-driven cavity at 0.8 oscillates and blows up within ~90 steps in
# the FP64 oracle and on the GPU alike, and is stable at 0.5 and below.
CFL = 0.4


@dataclass
class Problem:
    name: str
    case: M.Case
    gas: Gas
    cfl: float
    vs_maxlevel: int = 0

    def dt(self) -> float:
        """Δt_ξ of Status (src/Solver/Types.jl:509-520): CFL * min_d(ds_finest / U_d),
        U_d = max|u| - half of the finest velocity cell."""
        c = self.case
        ds = [(c.geometry[2 * d + 1] - c.geometry[2 * d]) / c.trees_num[d] / 2 ** c.max_level
              for d in range(c.dim)]
        q = c.quadrature
        U = [max(q[2 * d + 1], abs(q[2 * d])) - (q[2 * d + 1] - q[2 * d]) / c.vs_trees_num[d]
             / 2 ** self.vs_maxlevel / 2 for d in range(c.dim)]
        return self.cfl * min(ds[d] / U[d] for d in range(c.dim))


def sod(scale: float = 1.0, max_level: int = 2, nv: int = 28, x_bc: int = M.BC_OUTFLOW) -> Problem:
    """x_bc: the boundary kind of both x ends (UniformOutflow as in rp_1D.jl:45, or
    InterpolatedOutflow, CAIDVM.jl:71-94)."""
    tx = max(4, int(round(128 * scale)))
    ty = 4

    def ic(x):
        return [1.0, 0.0, 0.0, 0.5] if x[0] < 0.5 else [0.125, 0.0, 0.0, 0.625]

    def refine(mid, ds, L):
        # pre-refinement around the density jump (the reference refines on the gradient)
        return abs(mid[0] - 0.5) < (3.0 - L) * ds[0] * 2.0

    case = M.Case(
        dim=2, geometry=[0.0, 1.0, 0.0, 0.1], trees_num=[tx, ty], max_level=max_level,
        quadrature=[-5.0, 5.0, -5.0, 5.0], vs_trees_num=[nv, nv],
        domain_bc=[(x_bc, None), (x_bc, None), (M.BC_PERIOD, None), (M.BC_PERIOD, None)],
        ic=ic, refine=refine if max_level > 0 else None, gamma=5.0 / 3.0, K=1.0)
    return Problem("sod", case, Gas(Kn=1e-2, K=1.0, omega=0.81, omega_r=0.81), cfl=CFL)


def collision(center: float = 0.5, scale: float = 0.125, max_level: int = 1, nv: int = 12) -> Problem:
    """Two streams meeting in a tube ([0,1]x[0,0.1], outflow in x, periodic in y): left
    [1, 0.8, 0, 0.5], right [0.5, -0.8, 0, 0.8] with the jump at x = 0.47 (inside a tree, so
    the children of one parent can sit on either side), refinement around x = center, and per
    state a velocity grid refined by one level around its bulk velocity -- two grids each
    finer than the other somewhere.  Moving `center` gives a second mesh of the same case
    with cells kept, refined and coarsened (the adaptation tests)."""
    tx = max(4, int(round(128 * scale)))

    def ic(x):
        return [1.0, 0.8, 0.0, 0.5] if x[0] < 0.47 else [0.5, -0.8, 0.0, 0.8]

    def refine(mid, ds, L):
        return abs(mid[0] - center) < 2.0 * ds[0]

    case = M.Case(
        dim=2, geometry=[0.0, 1.0, 0.0, 0.1], trees_num=[tx, 4], max_level=max_level,
        quadrature=[-5.0, 5.0, -5.0, 5.0], vs_trees_num=[nv, nv],
        domain_bc=[(M.BC_OUTFLOW, None), (M.BC_OUTFLOW, None), (M.BC_PERIOD, None), (M.BC_PERIOD, None)],
        ic=ic, refine=refine if max_level > 0 else None, vgrid_fn=lambda prim: tuple(prim), vs_maxlevel=1,
        gamma=5.0 / 3.0, K=1.0)
    return Problem("collision", case, Gas(Kn=1e-2, K=1.0, omega=0.81, omega_r=0.81), cfl=CFL, vs_maxlevel=1)


def couette(n: int = 16, nv: int = 16) -> Problem:
    case = M.Case(
        dim=2, geometry=[-0.5, 0.5, -0.5, 0.5], trees_num=[n, n], max_level=0,
        quadrature=[-5.0, 5.0, -5.0, 5.0], vs_trees_num=[nv, nv],
        domain_bc=[(M.BC_MAXWELL, [1.0, 0.0, 0.0, 1.0]),
                   (M.BC_MAXWELL, [1.0, math.sqrt(5.0 / 6.0), 0.0, 1.0]),
                   (M.BC_PERIOD, None), (M.BC_PERIOD, None)],
        ic=lambda x: [1.0, 0.0, 0.0, 1.0], K=0.0)
    return Problem("couette", case, Gas(Kn=0.075, K=0.0, omega=0.81, omega_r=0.81), cfl=0.5)


def cavity(n: int = 32, nv: int = 24, levels: int = 0, Kn: float = 0.075, lid: float = 0.15) -> Problem:
    def refine(mid, ds, L):
        # refine along the walls
        m = min(mid[0], 1 - mid[0], mid[1], 1 - mid[1])
        return m < 2.0 * ds[0]

    case = M.Case(
        dim=2, geometry=[0.0, 1.0, 0.0, 1.0], trees_num=[n, n], max_level=levels,
        quadrature=[-6.0, 6.0, -6.0, 6.0], vs_trees_num=[nv, nv],
        domain_bc=[(M.BC_MAXWELL, [1.0, 0.0, 0.0, 1.0]), (M.BC_MAXWELL, [1.0, 0.0, 0.0, 1.0]),
                   (M.BC_MAXWELL, [1.0, 0.0, 0.0, 1.0]), (M.BC_MAXWELL, [1.0, lid, 0.0, 1.0])],
        ic=lambda x: [1.0, 0.0, 0.0, 1.0], refine=refine if levels > 0 else None, K=1.0)
    return Problem("cavity", case, Gas(Kn=Kn, K=1.0, omega=0.81, omega_r=0.81), cfl=CFL)


def cylinder(scale: float = 1.0, max_level: int = 3, nv: int = 48, vs_levels: int = 2,
             Ma: float = 5.0, Kn: float = 0.1, ubins: int = 4) -> Problem:
    n = max(8, int(round(64 * scale)))
    L = 8.0
    Uinf = Ma * math.sqrt(5.0 / 6.0)
    R = 1.0

    def ic(x):
        # cylinder_buffer_IC (example/cylinder/cylinder_udf.jl): a 1-wide buffer at the wall
        r = math.hypot(x[0], x[1])
        if r > R + 1.0:
            return [1.0, Uinf, 0.0, 1.0]
        return [1.0, (r - R) * Uinf, 0.0, 1.0]

    def refine(mid, ds, lev):
        r = math.hypot(mid[0], mid[1])
        d = abs(r - R)
        reach = [4.0, 2.2, 1.2][min(lev, 2)]
        return d < reach + 0.5 * math.hypot(ds[0], ds[1])

    def vgrid_key(prim):
        if vs_levels == 0:
            return None
        # bin the bulk speed so neighbouring cells share a handful of grids
        u = prim[1]
        b = round(u / Uinf * (ubins - 1))
        return (1.0, b * Uinf / (ubins - 1), 0.0, 1.0)

    case = M.Case(
        dim=2, geometry=[-L, L, -L, L], trees_num=[n, n], max_level=max_level,
        quadrature=[-15.0, 15.0, -15.0, 15.0], vs_trees_num=[nv, nv],
        domain_bc=[(M.BC_INFLOW, [1.0, Uinf, 0.0, 1.0]), (M.BC_OUTFLOW, None),
                   (M.BC_OUTFLOW, None), (M.BC_OUTFLOW, None)],
        ic=ic, refine=refine, circle=([0.0, 0.0], R, [1.0, 0.0, 0.0, 1.0]),
        vgrid_fn=vgrid_key, vs_maxlevel=vs_levels, K=1.0)
    return Problem("cylinder", case, Gas(Kn=Kn, K=1.0, omega=0.81, omega_r=0.81), cfl=CFL,
                   vs_maxlevel=vs_levels)


def build(problem: Problem):
    topo, state = M.build_topology(problem.case)
    return topo, state


def box3d(n=(6, 4, 4), nv: int = 8, levels: int = 1, Kn: float = 0.05) -> Problem:
    """3D one-distribution box: a density/temperature jump in x, outflow in x, periodic in
    y and z, optional refinement around the jump (exercises 3D hanging faces)."""
    def ic(x):
        return [1.0, 0.1, 0.0, 0.0, 0.5] if x[0] < 0.5 else [0.5, 0.1, 0.0, 0.0, 0.8]

    def refine(mid, ds, L):
        return abs(mid[0] - 0.5) < 1.2 * ds[0]

    case = M.Case(
        dim=3, geometry=[0.0, 1.0, 0.0, 1.0, 0.0, 1.0], trees_num=list(n), max_level=levels,
        quadrature=[-5.0, 5.0, -5.0, 5.0, -5.0, 5.0], vs_trees_num=[nv, nv, nv],
        domain_bc=[(M.BC_OUTFLOW, None), (M.BC_OUTFLOW, None), (M.BC_PERIOD, None), (M.BC_PERIOD, None),
                   (M.BC_PERIOD, None), (M.BC_PERIOD, None)],
        ic=ic, refine=refine if levels > 0 else None, K=0.0)
    return Problem("box3d", case, Gas(Kn=Kn, K=0.0, omega=0.81, omega_r=0.81), cfl=CFL)


def sphere(scale: float = 1.0, max_level: int = 2, nv: int = 24, Ma: float = 3.0, Kn: float = 0.05,
           reach: Tuple[float, float] = (1.8, 1.0)) -> Problem:
    """3D Ma 3 / Kn 0.05 flow past a diffuse isothermal sphere of radius 1 on [-6,6]^3,
    32^3 trees (scaled), 2 levels near the wall, uniform 24^3 velocity grid on [-10,10]^3.
    ``reach``: distance from the wall within which level 0 / level 1 cells are refined
    (``sphere_config`` widens it to the ~2e5 cells of the benchmark configuration)."""
    n = max(6, int(round(32 * scale)))
    Uinf = Ma * math.sqrt(5.0 / 6.0)
    R = 1.0

    def ic(x):
        r = math.sqrt(x[0] ** 2 + x[1] ** 2 + x[2] ** 2)
        if r > R + 1.0:
            return [1.0, Uinf, 0.0, 0.0, 1.0]
        return [1.0, (r - R) * Uinf, 0.0, 0.0, 1.0]

    def refine(mid, ds, lev):
        r = math.sqrt(mid[0] ** 2 + mid[1] ** 2 + mid[2] ** 2)
        rr = reach[min(lev, 1)]
        return abs(r - R) < rr + 0.5 * math.sqrt(ds[0] ** 2 + ds[1] ** 2 + ds[2] ** 2)

    case = M.Case(
        dim=3, geometry=[-6.0, 6.0, -6.0, 6.0, -6.0, 6.0], trees_num=[n, n, n], max_level=max_level,
        quadrature=[-10.0, 10.0, -10.0, 10.0, -10.0, 10.0], vs_trees_num=[nv, nv, nv],
        domain_bc=[(M.BC_INFLOW, [1.0, Uinf, 0.0, 0.0, 1.0]), (M.BC_OUTFLOW, None),
                   (M.BC_OUTFLOW, None), (M.BC_OUTFLOW, None), (M.BC_OUTFLOW, None), (M.BC_OUTFLOW, None)],
        ic=ic, refine=refine, circle=([0.0, 0.0, 0.0], R, [1.0, 0.0, 0.0, 0.0, 1.0]), K=0.0)
    return Problem("sphere", case, Gas(Kn=Kn, K=0.0, omega=0.81, omega_r=0.81), cfl=CFL)


def sphere_config() -> Problem:
    """The 3D sphere at its benchmark size: 32^3 trees, 2 levels within 3.5 / 1.8 of the wall
    (about 2.1e5 cells), 24^3 velocity grid: about 2.9e9 phase cells, f 11.7 GB in FP32."""
    return sphere(scale=1.0, reach=(3.5, 1.8))
