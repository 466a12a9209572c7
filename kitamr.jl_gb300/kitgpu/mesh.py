"""Synthetic forests and the reference-shaped flattened topology.

KitAMR.jl builds its physical mesh with p4est and its face list with a p4est face
iteration (src/Solver/Initialize.jl:5-158); neither p4est nor Julia is available to
this package's tests, so this module generates the same kind of data on the host:

* a 2:1-balanced quadtree/octree over a brick of trees (periodic or not),
* per-cell velocity grids in the reference's depth-first leaf order
  (src/Velocity_space/Initialize.jl:9-37, src/Velocity_space/Rebuild.jl:44-85),
* neighbour lists with the reference's states {0, 1, 2^(D-1), -1}
  (src/Mesh/Neighbor.jl:3-69, src/Physical_space/Types.jl:6-9),
* immersed-boundary classification for a circle/sphere, SolidNeighbor records
  with the intersect point and normal (src/Boundary/Circle.jl:33-62) and the
  velocity cut cells of src/Velocity_space/Cut_cell.jl:13-81,
* the face list exactly as initialize_full_face! / initialize_hanging_face! /
  initialize_domain_face! would emit it on one rank, with HangingFace sub-faces
  expanded (src/Solver/Initialize.jl:45-124, src/Flux/Flux.jl:37-59,84-89).

The output is a dict of numpy arrays whose names and meaning match ``kg_topology``
in include/kitgpu.h.  A Julia caller fills the same arrays from its own objects.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from fractions import Fraction
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

NBR_NONE = -(2 ** 31)
NBR_INSIDE = -(2 ** 31) + 1
FACE_INNER, FACE_DOMAIN = 0, 1
BC_MAXWELL, BC_INFLOW, BC_OUTFLOW, BC_INTERP, BC_PERIOD = 0, 1, 2, 3, 99

# refine midpoint table RMT (src/Abstract/Types.jl:10): children in x-fastest Z order
def _rmt(dim: int) -> List[Tuple[int, ...]]:
    out = []
    for c in range(2 ** dim):
        out.append(tuple(1 if (c >> d) & 1 else -1 for d in range(dim)))
    return out


def wall(w: int) -> int:
    return -1 - w


# --------------------------------------------------------------------------
# velocity grids
# --------------------------------------------------------------------------
@dataclass
class VGrid:
    level: np.ndarray      # int8 [nv]
    weight: np.ndarray     # f64 [nv]
    midpoint: np.ndarray   # f64 [nv, dim]

    @property
    def nv(self) -> int:
        return int(self.level.shape[0])

    def key(self) -> bytes:
        return self.level.tobytes() + self.midpoint.tobytes()


def uniform_vgrid(dim: int, quadrature: Sequence[float], vs_trees_num: Sequence[int]) -> VGrid:
    """Root lattice of initialize_vs_data (Velocity_space/Initialize.jl:9-37): midpoints of
    ``vs_trees_num[d]`` equal cells per dimension, the first dimension varying fastest
    (Iterators.product order), weight = product of root sizes (midpoint rule)."""
    axes = []
    ds = []
    for d in range(dim):
        lo, hi, n = Fraction(quadrature[2 * d]), Fraction(quadrature[2 * d + 1]), int(vs_trees_num[d])
        step = (hi - lo) / n
        ds.append(float(step))
        axes.append([float(lo + step * (k + Fraction(1, 2))) for k in range(n)])
    grids = np.meshgrid(*axes, indexing="ij")
    nv = int(np.prod(vs_trees_num))
    mid = np.empty((nv, dim))
    for d in range(dim):
        mid[:, d] = grids[d].reshape(-1, order="F")
    w = float(np.prod(ds))
    return VGrid(np.zeros(nv, np.int8), np.full(nv, w), mid)


def refine_vgrid(g: VGrid, flags: np.ndarray, root_ds: Sequence[float]) -> VGrid:
    """Streaming refinement of Velocity_space/Rebuild.jl:44-85: a flagged cell is
    replaced in place (depth-first) by its 2^D children in RMT order, weight / 2^D."""
    dim = g.midpoint.shape[1]
    nc = 2 ** dim
    rmt = _rmt(dim)
    lev, wt, mid = [], [], []
    for i in range(g.nv):
        if flags[i]:
            L = int(g.level[i])
            for c in range(nc):
                lev.append(L + 1)
                wt.append(g.weight[i] / nc)
                mid.append([g.midpoint[i, d] + 0.5 * (root_ds[d] / 2 ** (L + 1)) * rmt[c][d]
                            for d in range(dim)])
        else:
            lev.append(int(g.level[i]))
            wt.append(g.weight[i])
            mid.append(list(g.midpoint[i]))
    return VGrid(np.array(lev, np.int8), np.array(wt), np.array(mid, dtype=np.float64).reshape(-1, dim))


def coarsen_vgrid(g: VGrid, ok: np.ndarray, root_ds: Sequence[float], maxlevel: int) -> VGrid:
    """Streaming coarsening of Velocity_space/Rebuild.jl:96-163 (the grid part): walking the
    depth-first grid with the reference's alignment bookkeeping, a 2^D-aligned group of
    same-level siblings merges into its parent (level - 1, weight x 2^D, the midpoint half a
    child step from the first child's) when every member is willing (``ok``)."""
    dim = g.midpoint.shape[1]
    nc = 2 ** dim
    n = g.nv
    flag = [0.0] * (maxlevel + 1)
    lev, wt, mid = [], [], []

    def copy(i):
        lev.append(int(g.level[i])); wt.append(g.weight[i]); mid.append(list(g.midpoint[i]))
    index = 0
    while index < n:
        fl = int(g.level[index])
        if fl > 0:
            if (flag[fl] % 1 == 0.0 and index + nc - 1 < n
                    and all(int(g.level[index + k]) == fl for k in range(1, nc))):
                if all(bool(ok[index + k]) for k in range(nc)):
                    lev.append(fl - 1)
                    wt.append(g.weight[index] * nc)
                    mid.append([g.midpoint[index, d] + 0.5 * (root_ds[d] / 2 ** fl) for d in range(dim)])
                else:
                    for k in range(nc):
                        copy(index + k)
                index += nc
                for i in range(1, fl):
                    flag[i] += 1 / 2 ** (dim * (fl - i))
            else:
                copy(index)
                for i in range(1, fl + 1):
                    flag[i] += 1 / 2 ** (dim * (fl - i + 1))
                index += 1
        else:
            copy(index)
            index += 1
    return VGrid(np.array(lev, np.int8), np.array(wt), np.array(mid, dtype=np.float64).reshape(-1, dim))


def adapted_vgrid(dim, quadrature, vs_trees_num, prim, maxlevel: int, radius=(2.4, 1.2)) -> VGrid:
    """A velocity grid refined around the bulk velocity of ``prim`` (a static stand-in for
    the reference's velocity-space AMR, which stays on the host)."""
    g = uniform_vgrid(dim, quadrature, vs_trees_num)
    root_ds = [(quadrature[2 * d + 1] - quadrature[2 * d]) / vs_trees_num[d] for d in range(dim)]
    U = np.asarray(prim[1:1 + dim], dtype=np.float64)
    vth = 1.0 / math.sqrt(prim[-1])
    for lev in range(maxlevel):
        r = radius[min(lev, len(radius) - 1)] * vth
        dist = np.linalg.norm(g.midpoint - U[None, :], axis=1)
        flags = (dist < r) & (g.level == lev)
        g = refine_vgrid(g, flags, root_ds)
    return g


def vgrid_root_ds(quadrature, vs_trees_num, dim):
    return [(quadrature[2 * d + 1] - quadrature[2 * d]) / vs_trees_num[d] for d in range(dim)]


# --------------------------------------------------------------------------
# kinetic helpers used for initial states (lib/KitCore/2D.jl, 3D.jl, 2D2F.jl, 3D1F.jl)
# --------------------------------------------------------------------------
def get_conserved(prim, gamma):
    prim = np.asarray(prim, dtype=np.float64)
    dim = prim.shape[-1] - 2
    w = np.empty_like(prim)
    w[..., 0] = prim[..., 0]
    for d in range(dim):
        w[..., 1 + d] = prim[..., 0] * prim[..., 1 + d]
    u2 = sum(prim[..., 1 + d] ** 2 for d in range(dim))
    w[..., -1] = 0.5 * prim[..., 0] / prim[..., -1] / (gamma - 1.0) + 0.5 * prim[..., 0] * u2
    return w


def discrete_maxwell(mid: np.ndarray, prim, K: float) -> np.ndarray:
    """discrete_maxwell_2D2F (2D2F.jl:1-21) / discrete_maxwell_3D1F (3D1F.jl:1-13);
    returns [nv, ndf]."""
    dim = mid.shape[1]
    lam = prim[-1]
    c2 = sum((mid[:, d] - prim[1 + d]) ** 2 for d in range(dim))
    if dim == 2:
        h = prim[0] * (lam / math.pi) * np.exp(-lam * c2)
        b = h * K / (2.0 * lam)
        return np.stack([h, b], axis=1)
    m = prim[0] * (lam / math.pi) ** 1.5 * np.exp(-lam * c2)
    return m[:, None]


# --------------------------------------------------------------------------
# cut cells (Velocity_space/Cut_cell.jl:1-81)
# --------------------------------------------------------------------------
def _gaussian_area(pts: List[Tuple[float, float]]) -> float:
    area = 0.0
    n = len(pts)
    for i in range(n):
        j = (i + 1) % n
        area += pts[i][0] * pts[j][1] - pts[j][0] * pts[i][1]
    return 0.5 * abs(area)


def cut_rect(n, vertices):
    """Gas/solid areas of the rectangle ``vertices`` (anticlockwise from the lower-left
    corner) split by the line u.n = 0; restates cut_rect of Cut_cell.jl:13-77."""
    pts, idx = [], []
    i = 0
    xmin, xmax, ymin, ymax = vertices[0][0], vertices[1][0], vertices[0][1], vertices[2][1]
    y = -n[0] / n[1] * xmin
    if ymin < y < ymax:
        pts.append((xmin, y)); idx.append(8); i += 1
    y = -n[0] / n[1] * xmax
    if ymin < y < ymax:
        pts.append((xmax, y)); idx.append(4); i += 1
    x = -n[1] / n[0] * ymin
    if xmin < x < xmax:
        pts.append((x, ymin)); idx.append(2); i += 1
    x = -n[1] / n[0] * ymax
    if xmin < x < xmax:
        pts.append((x, ymax)); idx.append(6); i += 1
    CLP = [1, 3, 5, 7]
    clp = [k for k, v in enumerate(vertices) if v[0] * n[0] + v[1] * n[1] == 0.0]
    if len(clp) + i < 2:
        return False, 0.0, 0.0
    pts = pts + [tuple(v) for v in vertices]
    idx = idx + CLP
    order = sorted(range(len(idx)), key=lambda k: idx[k])  # labels are distinct
    idx = [idx[k] for k in order]
    pts = [pts[k] for k in order]
    online = {CLP[k] for k in clp}
    sel = [k for k, lab in enumerate(idx) if lab % 2 == 0 or lab in online]
    aid, bid = sel[0], sel[-1]
    A = pts[aid:bid + 1]
    l = (pts[bid][0] - pts[aid][0], pts[bid][1] - pts[aid][1])
    total = (xmax - xmin) * (ymax - ymin)
    if n[0] * l[1] - n[1] * l[0] < 0:
        gas = _gaussian_area(A)
        return True, gas, total - gas
    solid = _gaussian_area(A)
    return True, total - solid, solid


ANTIVT2 = [(-1, -1), (1, -1), (1, 1), (-1, 1)]


def cut_cells_2d(normal, g: VGrid, root_ds):
    """initialize_cutted_velocity_cell for 2D (Immersed_boundary.jl:226-249): the velocity
    cells crossed by u.n = 0 with their gas/solid areas."""
    if any(abs(x) < 1e-6 for x in normal):
        return [], [], []
    index, gas_w, solid_w = [], [], []
    for i in range(g.nv):
        ddu = [root_ds[d] / 2 ** int(g.level[i]) for d in range(2)]
        mid = g.midpoint[i]
        if abs(mid[0] * normal[0] + mid[1] * normal[1]) > 0.5 * math.hypot(ddu[0], ddu[1]):
            continue
        verts = [(0.5 * a * ddu[0] + mid[0], 0.5 * b * ddu[1] + mid[1]) for a, b in ANTIVT2]
        flag, gw, sw = cut_rect(normal, verts)
        if flag:
            index.append(i); gas_w.append(gw); solid_w.append(sw)
    return index, gas_w, solid_w


def _box_below_plane(n, lo, hi) -> float:
    """Volume of {x in [lo, hi] : n.x <= 0} (exact inclusion-exclusion over the box corners)."""
    dim = len(n)
    a, b = [], 0.0
    for d in range(dim):
        s = hi[d] - lo[d]
        ad = n[d] * s
        b -= n[d] * lo[d]
        if ad < 0:          # t -> 1 - t makes every coefficient non-negative
            b -= ad
            ad = -ad
        a.append(ad)
    amax = max(a) if a else 0.0
    act = [x for x in a if x > 1e-12 * max(amax, 1e-300)]
    vol = 1.0
    for d in range(dim):
        vol *= hi[d] - lo[d]
    k = len(act)
    if k == 0:
        return vol if b >= 0 else 0.0
    tot = 0.0
    for mask in range(1 << k):
        sa, bits = 0.0, 0
        for i in range(k):
            if (mask >> i) & 1:
                sa += act[i]
                bits += 1
        r = b - sa
        if r > 0:
            tot += (-1) ** bits * r ** k
    frac = tot / (math.factorial(k) * float(np.prod(act)))
    return vol * min(max(frac, 0.0), 1.0)


def _boxes_below_plane(n, lo, hi) -> np.ndarray:
    """_box_below_plane over many boxes at once (rows of lo / hi), the same arithmetic in the
    same order per box."""
    nb, dim = lo.shape
    s = hi - lo
    a = n[None, :] * s
    b = -(n[None, :] * lo)
    bsum = np.zeros(nb)
    for d in range(dim):
        bsum = bsum + b[:, d]
        neg = a[:, d] < 0
        bsum = np.where(neg, bsum - a[:, d], bsum)
    a = np.abs(a)
    vol = np.ones(nb)
    for d in range(dim):
        vol = vol * s[:, d]
    out = np.empty(nb)
    amax = np.max(a, axis=1)
    act = a > 1e-12 * np.maximum(amax, 1e-300)[:, None]
    full = np.all(act, axis=1)
    if np.any(full):
        # boxes with every coefficient active: the same sum over corners, term by term in
        # the scalar form's order, for all of them at once
        af, bf = a[full], bsum[full]
        tot = np.zeros(af.shape[0])
        for mask in range(1 << dim):
            sa = np.zeros(af.shape[0])
            bits = 0
            for i in range(dim):
                if (mask >> i) & 1:
                    sa = sa + af[:, i]
                    bits += 1
            r = bf - sa
            term = (-1) ** bits * np.power(r, float(dim))
            tot = np.where(r > 0, tot + term, tot)
        pr = np.ones(af.shape[0])
        for i in range(dim):
            pr = pr * af[:, i]
        frac = tot / (math.factorial(dim) * pr)
        out[full] = vol[full] * np.minimum(np.maximum(frac, 0.0), 1.0)
    for row in np.nonzero(~full)[0]:
        # the inclusion-exclusion sum is short (at most 2^dim terms): per box, as in the scalar form
        av = [float(x) for x, m in zip(a[row], act[row]) if m]
        k = len(av)
        bb = float(bsum[row])
        if k == 0:
            out[row] = vol[row] if bb >= 0 else 0.0
            continue
        tot = 0.0
        for mask in range(1 << k):
            sa, bits = 0.0, 0
            for i in range(k):
                if (mask >> i) & 1:
                    sa += av[i]
                    bits += 1
            r = bb - sa
            if r > 0:
                tot += (-1) ** bits * r ** k
        pr = 1.0
        for x in av:
            pr *= x
        frac = tot / (math.factorial(k) * pr)
        out[row] = vol[row] * min(max(frac, 0.0), 1.0)
    return out


def cut_cells_3d(normal, g: VGrid, root_ds):
    """3D counterpart of the cut-cell split (Immersed_boundary.jl:250-277): for each velocity
    cell crossed by u.n = 0, its gas (u.n < 0) and solid (u.n > 0) volumes.  The split is
    host geometry; the volumes come from an exact box / half-space formula.  The screening
    test runs over the whole grid at once; only the crossed cells get the volume formula."""
    if sum(1 for x in normal if abs(x) < 1e-6) > 1:
        return [], [], []
    n = np.asarray(normal, dtype=np.float64)
    lev = np.asarray(g.level, dtype=np.int64)
    ddu = np.stack([root_ds[d] / 2.0 ** lev for d in range(3)], axis=1)
    mid = np.asarray(g.midpoint, dtype=np.float64).reshape(-1, 3)
    proj = mid[:, 0] * n[0] + mid[:, 1] * n[1] + mid[:, 2] * n[2]
    half_diag = 0.5 * np.sqrt(ddu[:, 0] * ddu[:, 0] + ddu[:, 1] * ddu[:, 1] + ddu[:, 2] * ddu[:, 2])
    cand = np.nonzero(~(np.abs(proj) > half_diag))[0]
    if cand.size == 0:
        return [], [], []
    lo = mid[cand] - 0.5 * ddu[cand]
    hi = mid[cand] + 0.5 * ddu[cand]
    tot = ddu[cand, 0] * ddu[cand, 1] * ddu[cand, 2]
    gas = _boxes_below_plane(n, lo, hi)
    keep = (1e-12 * tot < gas) & (gas < tot * (1 - 1e-12))
    idx = cand[keep]
    return [int(i) for i in idx], [float(x) for x in gas[keep]], [float(x) for x in (tot - gas)[keep]]


def calc_intersect_sphere(f_mid, s_mid, center, radius, solid=True):
    """calc_intersect(::Sphere) of Boundary/Circle.jl:52-62 (as written: the normal keeps the
    donor's coordinates in the two tangential directions; the generated cases use center 0)."""
    r = radius
    dirs = [d for d in range(3) if abs(f_mid[d] - s_mid[d]) > 1e-12]
    dr = dirs[0]
    rm = [f_mid[d] - center[d] for d in range(3)]
    x = rm[(dr + 1) % 3]
    y = rm[(dr + 2) % 3]
    rz = math.sqrt(r * r - x * x - y * y)
    if abs((rz - rm[dr]) / (s_mid[dr] - f_mid[dr])) < 1:
        dz = rz - rm[dr]
    else:
        dz = -rz - rm[dr]
    ap = list(f_mid)
    nv = list(f_mid)
    ap[dr] = dz + f_mid[dr]
    nv[dr] = dz + rm[dr]
    den = r if solid else -r
    return ap, [v / den for v in nv]


def calc_intersect_circle(f_mid, s_mid, center, radius, solid=True):
    """calc_intersect(::Circle) of Boundary/Circle.jl:33-51 (the reference leaves the
    intersect point relative to the origin; the generated cases use center [0,0])."""
    r = radius
    if abs(f_mid[0] - s_mid[0]) < 1e-12:
        t = math.acos((f_mid[0] - center[0]) / r)
        if f_mid[1] > center[1]:
            ap = [r * math.cos(t), r * math.sin(t)]
        else:
            ap = [r * math.cos(t), -r * math.sin(t)]
    else:
        t = math.asin((f_mid[1] - center[1]) / r)
        if f_mid[0] > center[0]:
            ap = [r * math.cos(t), r * math.sin(t)]
        else:
            ap = [-r * math.cos(t), r * math.sin(t)]
    den = r if solid else -r
    return ap, [ap[0] / den, ap[1] / den]


# --------------------------------------------------------------------------
# physical forest
# --------------------------------------------------------------------------
@dataclass
class Case:
    dim: int
    geometry: Sequence[float]
    trees_num: Sequence[int]
    max_level: int
    quadrature: Sequence[float]
    vs_trees_num: Sequence[int]
    domain_bc: Sequence[Tuple[int, Optional[Sequence[float]]]]  # per faceid: (BC kind, bc prim)
    ic: Callable[[np.ndarray], Sequence[float]]
    refine: Optional[Callable[[np.ndarray, np.ndarray, int], bool]] = None
    circle: Optional[Tuple[Sequence[float], float, Sequence[float]]] = None  # center, radius, wall prim
    search_coeffi: float = 4.0
    vgrid_fn: Optional[Callable[[np.ndarray], Tuple]] = None  # cell prim -> grid key (hashable)
    vs_maxlevel: int = 0
    gamma: float = 5.0 / 3.0
    K: float = 1.0


def _morton(coords: Sequence[int], bits: int) -> int:
    code = 0
    dim = len(coords)
    for b in range(bits):
        for d in range(dim):
            code |= ((coords[d] >> b) & 1) << (b * dim + d)
    return code


def build_forest(case: Case):
    dim, L_max = case.dim, case.max_level
    tn = list(case.trees_num)
    geom = [Fraction(x) for x in case.geometry]
    periodic = [case.domain_bc[2 * d][0] == BC_PERIOD for d in range(dim)]

    def extent(L, d):
        return tn[d] * (1 << L)

    def h_exact(L, d):
        return (geom[2 * d + 1] - geom[2 * d]) / tn[d] / (1 << L)

    # centre coordinates are exact rationals rounded once; memoised per (level, index) along
    # each axis, since a coordinate repeats across the leaves of a row
    _coord: Dict[Tuple[int, int, int], float] = {}

    def coord(L, d, i):
        key = (L, d, i)
        v = _coord.get(key)
        if v is None:
            v = float(geom[2 * d] + h_exact(L, d) * (i + Fraction(1, 2)))
            _coord[key] = v
        return v

    def center(L, idx):
        return np.array([coord(L, d, idx[d]) for d in range(dim)])

    _ds: Dict[int, np.ndarray] = {}

    def dsv(L):
        v = _ds.get(L)
        if v is None:
            v = np.array([float(h_exact(L, d)) for d in range(dim)])
            _ds[L] = v
        return v.copy()

    leaves = set()
    for idx in np.ndindex(*tn):
        leaves.add((0,) + tuple(int(i) for i in idx))
    # refinement passes, coarse to fine
    if case.refine is not None:
        for L in range(L_max):
            cur = [lf for lf in leaves if lf[0] == L]
            for lf in cur:
                idx = lf[1:]
                if case.refine(center(L, idx), dsv(L), L):
                    leaves.remove(lf)
                    for c in range(2 ** dim):
                        leaves.add((L + 1,) + tuple(2 * idx[d] + ((c >> d) & 1) for d in range(dim)))

    def wrap(L, idx):
        out = list(idx)
        for d in range(dim):
            n = extent(L, d)
            if out[d] < 0 or out[d] >= n:
                if not periodic[d]:
                    return None
                out[d] %= n
        return tuple(out)

    # 2:1 face balance: a leaf whose face neighbour region holds leaves two or more
    # levels finer is refined, until no such leaf remains
    def covered(L, n):
        for l in range(L, -1, -1):
            if (l, *[x >> (L - l) for x in n]) in leaves:
                return True
        return False

    changed = True
    while changed:
        changed = False
        for lf in sorted(leaves, key=lambda x: x[0]):
            if lf not in leaves:
                continue
            L, idx = lf[0], lf[1:]
            need = False
            for d in range(dim):
                for s in (-1, 1):
                    n = list(idx); n[d] += s
                    n = wrap(L, n)
                    if n is None or covered(L, n):
                        continue
                    # region (L, n) is subdivided: its children adjacent to the face
                    # must be leaves, otherwise the face would be 1:4
                    want = 0 if s == 1 else 1
                    for c in range(2 ** dim):
                        if ((c >> d) & 1) != want:
                            continue
                        ch = (L + 1,) + tuple(2 * n[e] + ((c >> e) & 1) for e in range(dim))
                        if ch not in leaves:
                            need = True
                            break
                    if need:
                        break
                if need:
                    break
            if need:
                leaves.remove(lf)
                for c in range(2 ** dim):
                    leaves.add((L + 1,) + tuple(2 * idx[d] + ((c >> d) & 1) for d in range(dim)))
                changed = True

    # p4est-like order: trees row-major (x fastest), Morton inside a tree
    def order_key(lf):
        L, idx = lf[0], lf[1:]
        fine = [idx[d] << (L_max - L) for d in range(dim)]
        tree = [f >> L_max for f in fine]
        tlin = 0
        stride = 1
        for d in range(dim):
            tlin += tree[d] * stride
            stride *= tn[d]
        local = [f & ((1 << L_max) - 1) for f in fine]
        return (tlin, _morton(local, L_max))

    order = sorted(leaves, key=order_key)
    return order, center, dsv, wrap, periodic


def build_topology(case: Case, dtype_check: bool = True) -> Dict[str, np.ndarray]:
    dim = case.dim
    ndf = 2 if dim == 2 else 1
    order, center, dsv, wrap, periodic = build_forest(case)
    lid = {lf: i for i, lf in enumerate(order)}
    nleaf = len(order)
    mids = np.array([center(lf[0], lf[1:]) for lf in order]).reshape(nleaf, dim)
    dss = np.array([dsv(lf[0]) for lf in order]).reshape(nleaf, dim)
    levels = np.array([lf[0] for lf in order], np.int32)

    # ---- neighbour lists over leaves ------------------------------------
    nstate = np.zeros((nleaf, 2 * dim), np.int8)
    nlist: List[List[List[int]]] = [[[] for _ in range(2 * dim)] for _ in range(nleaf)]
    nwrap = np.zeros((nleaf, 2 * dim), bool)  # the face crosses a periodic boundary
    for i, lf in enumerate(order):
        L, idx = lf[0], lf[1:]
        for k in range(2 * dim):
            d, s = k // 2, (1 if k % 2 else -1)
            raw = list(idx); raw[d] += s
            n = wrap(L, raw)
            if n is None:
                nstate[i, k] = 0
                nlist[i][k] = [NBR_NONE]
                continue
            nwrap[i, k] = tuple(raw) != n
            if (L, *n) in lid:
                nstate[i, k] = 1
                nlist[i][k] = [lid[(L, *n)]]
            elif L > 0 and (L - 1, *[x >> 1 for x in n]) in lid:
                nstate[i, k] = -1
                nlist[i][k] = [lid[(L - 1, *[x >> 1 for x in n])]]
            else:
                nstate[i, k] = 2 ** (dim - 1)
                lst = []
                tdims = [e for e in range(dim) if e != d]
                for c in range(2 ** (dim - 1)):
                    ch = [0] * dim
                    ch[d] = 2 * n[d] + (1 if s == -1 else 0)
                    for b, e in enumerate(tdims):
                        ch[e] = 2 * n[e] + ((c >> b) & 1)
                    key = (L + 1, *ch)
                    if key not in lid:
                        raise RuntimeError("forest is not 2:1 balanced")
                    lst.append(lid[key])
                nlist[i][k] = lst

    # ---- immersed boundary classification ---------------------------------
    kind = np.zeros(nleaf, np.int8)  # 0 fluid, 1 solid ghost, 2 inside solid
    if case.circle is not None:
        c0, R, _wbc = case.circle
        c0 = np.asarray(c0, dtype=np.float64)
        for i in range(nleaf):
            inside = np.linalg.norm(mids[i] - c0) <= R
            if not inside:
                continue
            flag = 0
            for d in range(dim):
                for s in (-1, 1):
                    p = mids[i].copy(); p[d] += s * dss[i, d]
                    flag += 1 if np.linalg.norm(p - c0) > R else -1
            kind[i] = 1 if abs(flag) != 2 * dim else 2

    cell_of_leaf = -np.ones(nleaf, np.int64)
    cells = [i for i in range(nleaf) if kind[i] != 2]
    for ci, i in enumerate(cells):
        cell_of_leaf[i] = ci
    ncell = len(cells)
    bound_enc = np.array([-1 if kind[i] == 1 else 0 for i in cells], np.int32)

    def ref_of(leaf_ref):
        if leaf_ref == NBR_NONE:
            return NBR_NONE
        c = cell_of_leaf[leaf_ref]
        return NBR_INSIDE if c < 0 else int(c)

    cnbr = [[[ref_of(x) for x in nlist[i][k]] for k in range(2 * dim)] for i in cells]

    # ---- velocity grids ---------------------------------------------------
    prims = np.array([case.ic(mids[i]) for i in cells], dtype=np.float64).reshape(ncell, dim + 2)
    grids: List[VGrid] = []
    gkey: Dict = {}
    cell_grid = np.zeros(ncell, np.int32)
    root_ds = vgrid_root_ds(case.quadrature, case.vs_trees_num, dim)
    for c in range(ncell):
        key = case.vgrid_fn(prims[c]) if case.vgrid_fn is not None else None
        if key not in gkey:
            if key is None:
                g = uniform_vgrid(dim, case.quadrature, case.vs_trees_num)
            else:
                g = adapted_vgrid(dim, case.quadrature, case.vs_trees_num, list(key), case.vs_maxlevel)
            gkey[key] = len(grids)
            grids.append(g)
        cell_grid[c] = gkey[key]

    # ---- solid neighbours (initialize_solid_neighbor!, Immersed_boundary.jl:282-305)
    walls = []
    if case.circle is not None:
        c0, R, wbc = case.circle
        for c in range(ncell):
            if bound_enc[c] < 0:
                continue
            for k in range(2 * dim):
                r0 = cnbr[c][k][0]
                if r0 < 0 or bound_enc[r0] >= 0:
                    continue
                s = r0
                bound_enc[c] = -bound_enc[s]
                g = grids[cell_grid[c]]
                if dim == 2:
                    ap, nrm = calc_intersect_circle(mids[cells[c]], mids[cells[s]], c0, R, True)
                    cidx, cgw, csw = cut_cells_2d(nrm, g, root_ds)
                else:
                    ap, nrm = calc_intersect_sphere(mids[cells[c]], mids[cells[s]], c0, R, True)
                    cidx, cgw, csw = cut_cells_3d(nrm, g, root_ds)
                walls.append(dict(donor=c, solid=s, faceid=k, aux=ap, normal=nrm, bc=list(wbc),
                                  cut=cidx, gw=cgw, sw=csw))
                cnbr[c][k][0] = wall(len(walls) - 1)

    # ---- faces (initialize_faces!, Solver/Initialize.jl:5-124, one rank) ---
    def cell_mid(r):
        if r >= 0:
            return mids[cells[r]]
        w = -1 - r
        return mids[cells[walls[w]["solid"]]]

    def cell_ds(r):
        if r >= 0:
            return dss[cells[r]]
        return dss[cells[walls[-1 - r]["solid"]]]

    def is_fluid_psdata(r):
        return r >= 0 and bound_enc[r] >= 0

    def face_area(ds_, d):
        if dim == 2:
            return ds_[1 - d]
        a, b = [e for e in range(3) if e != d]
        return ds_[a] * ds_[b]

    def rot_of(k):  # get_rot(faceid) with faceid = k + 1
        return 1.0 if k % 2 == 0 else -1.0

    F = dict(kind=[], dir=[], rot=[], area=[], mid=[], here=[], there=[], there_mid=[], bck=[], bc=[])

    def emit(kd, d, rot, area, mid, here, there, there_mid, bck=0, bc=None):
        F["kind"].append(kd); F["dir"].append(d); F["rot"].append(rot); F["area"].append(area)
        F["mid"].append(list(mid)); F["here"].append(here); F["there"].append(there)
        F["there_mid"].append(list(there_mid) if there_mid is not None else [0.0] * dim)
        F["bck"].append(bck); F["bc"].append(list(bc) if bc is not None else [0.0] * (dim + 2))

    for i, lf in enumerate(order):
        ci = cell_of_leaf[i]
        for k in range(2 * dim):
            d = k // 2
            st = nstate[i, k]
            if st == 0:
                if ci < 0:
                    continue
                bkind, bcv = case.domain_bc[k]
                rot = rot_of(k)
                mid = mids[i].copy(); mid[d] -= 0.5 * rot * dss[i, d]
                emit(FACE_DOMAIN, d, rot, rot * face_area(dss[i], d), mid, int(ci), NBR_NONE, None, bkind, bcv)
                continue
            if st == 1 and k % 2 == 1:
                # full face, emitted once from the lower cell's +face (side A)
                if ci < 0:
                    continue
                base, kk = int(ci), k
                if bound_enc[base] < 0:
                    nb = cnbr[base][kk][0]
                    if not is_fluid_psdata(nb):
                        continue
                    base, kk = nb, (kk - 1 if kk % 2 == 1 else kk + 1)
                rot = rot_of(kk)
                bmid = mids[cells[base]]; bds = dss[cells[base]]
                mid = bmid.copy(); mid[d] -= 0.5 * rot * bds[d]
                there = cnbr[base][kk][0]
                crosses = nwrap[cells[base], kk]
                if crosses:
                    tmid = mid.copy(); tmid[d] -= 0.5 * rot * bds[d]
                else:
                    tmid = cell_mid(there)
                emit(FACE_INNER, d, rot, face_area(bds, d) * rot, mid, base, there, tmid)
                continue
            if st == 2 ** (dim - 1):
                # hanging face, emitted by the coarse side
                if ci < 0:
                    continue
                base = int(ci)
                rot = rot_of(k)
                nlst = cnbr[base][k]
                if bound_enc[base] < 0:
                    ids = [r for r in nlst if is_fluid_psdata(r)]
                    if not ids:
                        continue
                    kk = k - 1 if k % 2 == 1 else k + 1
                    rr = rot_of(kk)
                    for r in ids:
                        mid = mids[cells[r]].copy(); mid[d] -= 0.5 * rr * dss[cells[r], d]
                        emit(FACE_INNER, d, rr, face_area(dss[cells[r]], d) * rr, mid, r, base,
                             mids[cells[base]])
                    continue
                crosses = nwrap[i, k]
                bmid = mids[i]; bds = dss[i]
                for r in nlst:
                    mid = cell_mid(r).copy(); mid[d] = bmid[d] - 0.5 * rot * bds[d]
                    if crosses:
                        tmid = mid.copy(); tmid[d] -= 0.5 * rot * cell_ds(r)[d]
                    else:
                        tmid = cell_mid(r)
                    emit(FACE_INNER, d, rot, face_area(bds, d) / 2 ** (dim - 1) * rot, mid, base, r, tmid)

    # ---- pack ---------------------------------------------------------------
    nflat = []
    noff = [0]
    nst = np.zeros(ncell * 2 * dim, np.int8)
    for c in range(ncell):
        for k in range(2 * dim):
            nflat.extend(cnbr[c][k])
            noff.append(len(nflat))
            nst[c * 2 * dim + k] = nstate[cells[c], k]
    goff = np.zeros(len(grids) + 1, np.int64)
    for g, gg in enumerate(grids):
        goff[g + 1] = goff[g] + gg.nv
    vmid = np.concatenate([gg.midpoint.reshape(-1, order="F") for gg in grids])
    cut_off = [0]
    cut_idx, cut_gw, cut_sw = [], [], []
    for w in walls:
        cut_idx += w["cut"]; cut_gw += w["gw"]; cut_sw += w["sw"]
        cut_off.append(len(cut_idx))
    nw = len(walls)
    topo = dict(
        dim=dim, ndf=ndf,
        n_grids=len(grids), grid_off=goff,
        vs_level=np.concatenate([g.level for g in grids]).astype(np.int8),
        vs_weight=np.concatenate([g.weight for g in grids]),
        vs_midpoint=vmid,
        n_cells=ncell,
        cell_bound_enc=bound_enc,
        cell_level=levels[cells].astype(np.int32),
        cell_grid=cell_grid,
        cell_midpoint=np.ascontiguousarray(mids[cells]).reshape(-1),
        cell_ds=np.ascontiguousarray(dss[cells]).reshape(-1),
        nbr_state=nst, nbr_off=np.array(noff, np.int32), nbr_ref=np.array(nflat, np.int32),
        n_walls=nw,
        wall_donor=np.array([w["donor"] for w in walls], np.int32),
        wall_solid=np.array([w["solid"] for w in walls], np.int32),
        wall_faceid=np.array([w["faceid"] for w in walls], np.int32),
        wall_aux_point=np.array([w["aux"] for w in walls], np.float64).reshape(-1),
        wall_normal=np.array([w["normal"] for w in walls], np.float64).reshape(-1),
        wall_bc=np.array([w["bc"] for w in walls], np.float64).reshape(-1),
        wall_cut_off=np.array(cut_off, np.int32),
        wall_cut_index=np.array(cut_idx, np.int32),
        wall_cut_gas_w=np.array(cut_gw, np.float64),
        wall_cut_solid_w=np.array(cut_sw, np.float64),
        n_faces=len(F["kind"]),
        face_kind=np.array(F["kind"], np.int8), face_dir=np.array(F["dir"], np.int8),
        face_rot=np.array(F["rot"], np.float64), face_area=np.array(F["area"], np.float64),
        face_midpoint=np.array(F["mid"], np.float64).reshape(-1),
        face_here=np.array(F["here"], np.int32), face_there=np.array(F["there"], np.int32),
        face_there_midpoint=np.array(F["there_mid"], np.float64).reshape(-1),
        face_bc_kind=np.array(F["bck"], np.int8), face_bc=np.array(F["bc"], np.float64).reshape(-1),
        # per cell its forest leaf (level, index...): not part of kg_topology, it lets two
        # meshes of one case be matched cell by cell (adapt_sources)
        cell_leaf=np.array([order[i] for i in cells], np.int64).reshape(ncell, 1 + dim),
        # per cell its position among all leaves (InsideSolidData included), and their count:
        # the quadrant order of the reference's per-rank checkpoint arrays
        cell_quad=np.array(cells, np.int32), n_quads=nleaf,
    )
    # initial state (initialize_ps!, Solver/Initialize.jl:343-380): w from prim, f = Maxwellian
    # (cells of one grid and one initial state share their block: a freestream is one block)
    K = case.K
    fcache: Dict = {}
    fblocks = []
    for c in range(ncell):
        key = (int(cell_grid[c]), prims[c].tobytes())
        blk = fcache.get(key)
        if blk is None:
            g = grids[cell_grid[c]]
            blk = discrete_maxwell(g.midpoint, prims[c], K).reshape(-1, order="F")
            fcache[key] = blk
        fblocks.append(blk)
    state = dict(f=np.concatenate(fblocks), w=get_conserved(prims, case.gamma).reshape(-1),
                 prim=prims.reshape(-1).copy())
    return topo, state


def phase_cells(topo) -> int:
    """Σ velocity cells over cells with bound_enc >= 0 (check_vs_num, IO/Check.jl:98-108)."""
    goff = topo["grid_off"]
    nv = (goff[1:] - goff[:-1])[topo["cell_grid"]]
    return int(nv[topo["cell_bound_enc"] >= 0].sum())


def f_offsets(topo) -> np.ndarray:
    goff = topo["grid_off"]
    nv = (goff[1:] - goff[:-1])[topo["cell_grid"]]
    off = np.zeros(topo["n_cells"] + 1, np.int64)
    off[1:] = np.cumsum(nv * topo["ndf"])
    return off


# --------------------------------------------------------------------------
# adaptation between two meshes of one case (the replacement callbacks' record)
# --------------------------------------------------------------------------
from .abi import ADAPT_SRC, KG_ADAPT_COARSEN as ADAPT_COARSEN, KG_ADAPT_KEEP as ADAPT_KEEP  # noqa: E402
from .abi import KG_ADAPT_REFINE as ADAPT_REFINE  # noqa: E402


def adapt_sources(old: Dict, new: Dict) -> np.ndarray:
    """Per cell of ``new``, where ps_replace! (Physical_space/AMR.jl:633-703) takes its
    state from in ``old`` (kg_adapt_src records), by matching the meshes' leaves: the same
    leaf (KEEP), a leaf below an old one (REFINE, child numbers in RMT order from the old
    leaf down), or the parent of 2^dim old leaves (COARSEN, children in RMT order)."""
    dim = int(new["dim"])
    lo = {tuple(int(v) for v in x): i for i, x in enumerate(old["cell_leaf"])}
    out = np.zeros(int(new["n_cells"]), ADAPT_SRC)
    for c, x in enumerate(new["cell_leaf"]):
        lf = tuple(int(v) for v in x)
        L, idx = lf[0], lf[1:]
        if lf in lo:
            out[c]["kind"] = ADAPT_KEEP
            out[c]["src"][0] = lo[lf]
            continue
        done = False
        for up in range(1, L + 1):
            anc = (L - up, *[v >> up for v in idx])
            if anc in lo:
                if up > 8:
                    raise ValueError("refinement deeper than 8 levels in one adaptation")
                out[c]["kind"] = ADAPT_REFINE
                out[c]["depth"] = up
                out[c]["src"][0] = lo[anc]
                for s in range(1, up + 1):
                    out[c]["path"][s - 1] = sum(((idx[d] >> (up - s)) & 1) << d for d in range(dim))
                done = True
                break
        if done:
            continue
        ch = [(L + 1, *[2 * idx[d] + ((q >> d) & 1) for d in range(dim)]) for q in range(2 ** dim)]
        if all(k in lo for k in ch):
            out[c]["kind"] = ADAPT_COARSEN
            out[c]["src"][:2 ** dim] = [lo[k] for k in ch]
            continue
        raise ValueError(f"cell {c} (leaf {lf}) is neither kept, refined nor a one-level coarsening")
    return out


def adapt_grids(old: Dict, new: Dict, src: np.ndarray) -> Dict:
    """``new`` with the velocity grids ps_replace! gives its cells: a kept or refined cell
    keeps its source's grid (ps_copy), a coarsened one takes the grid of its first child with
    the fewest velocity cells (ps_merge).  The grid table becomes ``old``'s.  A wall's cut
    cells were computed on its donor's grid in ``new``, so every donor must keep that grid."""
    dim = int(new["dim"])
    out = dict(new)
    for k in ("n_grids", "grid_off", "vs_level", "vs_weight", "vs_midpoint"):
        out[k] = old[k]
    goff = np.asarray(old["grid_off"])
    nvg = goff[1:] - goff[:-1]
    ocg = np.asarray(old["cell_grid"])
    cg = np.empty(int(new["n_cells"]), np.int32)
    for c, r in enumerate(src):
        if r["kind"] == ADAPT_COARSEN:
            ch = r["src"][:2 ** dim]
            cg[c] = ocg[ch[int(np.argmin(nvg[ocg[ch]]))]]
        else:
            cg[c] = ocg[r["src"][0]]
    out["cell_grid"] = cg

    def grid_arrays(t, g):
        o = np.asarray(t["grid_off"])
        a, b = int(o[g]), int(o[g + 1])
        return (np.asarray(t["vs_level"])[a:b], np.asarray(t["vs_weight"])[a:b],
                np.asarray(t["vs_midpoint"])[a * dim:b * dim])
    for dn in np.unique(np.asarray(new["wall_donor"], np.int64)):
        ga, gb = grid_arrays(old, int(cg[dn])), grid_arrays(new, int(new["cell_grid"][dn]))
        if not all(np.array_equal(x, y) for x, y in zip(ga, gb)):
            raise ValueError(f"wall donor {dn} changes its velocity grid; its cut cells would not match")
    return out


def cell_vgrid(topo: Dict, cell: int) -> VGrid:
    """The velocity grid of ``cell`` in a topology."""
    dim = int(topo["dim"])
    g = int(topo["cell_grid"][cell])
    o = np.asarray(topo["grid_off"])
    a, b = int(o[g]), int(o[g + 1])
    return VGrid(np.asarray(topo["vs_level"])[a:b].astype(np.int8), np.asarray(topo["vs_weight"])[a:b].copy(),
                 np.asarray(topo["vs_midpoint"])[a * dim:b * dim].reshape(dim, b - a).T.copy())


def with_cell_vgrids(topo: Dict, grids: Dict[int, VGrid]) -> Dict:
    """``topo`` with new velocity grids for some cells (a velocity-space adaptation): grids are
    appended to the grid table (or shared with an equal one).  A wall donor may not change its
    grid: its wall's cut cells index that grid."""
    dim = int(topo["dim"])
    out = dict(topo)
    donors = set(int(x) for x in np.asarray(topo.get("wall_donor", np.zeros(0, np.int32))))
    level = [np.asarray(topo["vs_level"])]
    weight = [np.asarray(topo["vs_weight"])]
    mid = [np.asarray(topo["vs_midpoint"])]
    goff = list(np.asarray(topo["grid_off"], np.int64))
    known = {}
    for g in range(int(topo["n_grids"])):
        a, b = goff[g], goff[g + 1]
        known[level[0][a:b].tobytes() + mid[0][a * dim:b * dim].tobytes()] = g
    cg = np.asarray(topo["cell_grid"], np.int32).copy()
    for c, vg in grids.items():
        key = vg.level.astype(np.int8).tobytes() + vg.midpoint.reshape(-1, order="F").tobytes()
        g = known.get(key)
        if g is None:
            g = len(goff) - 1
            known[key] = g
            level.append(vg.level.astype(np.int8)); weight.append(vg.weight)
            mid.append(vg.midpoint.reshape(-1, order="F"))
            goff.append(goff[-1] + vg.nv)
        if c in donors and g != cg[c]:
            raise ValueError(f"wall donor {c} changes its velocity grid; its cut cells would not match")
        cg[c] = g
    out.update(n_grids=len(goff) - 1, grid_off=np.array(goff, np.int64),
               vs_level=np.concatenate(level).astype(np.int8), vs_weight=np.concatenate(weight),
               vs_midpoint=np.concatenate(mid), cell_grid=cg)
    return out


def vs_sources(topo: Dict) -> np.ndarray:
    """One KG_ADAPT_VS record per cell (each cell its own source)."""
    from .abi import KG_ADAPT_VS
    out = np.zeros(int(topo["n_cells"]), ADAPT_SRC)
    out["kind"] = KG_ADAPT_VS
    out["src"][:, 0] = np.arange(int(topo["n_cells"]))
    return out
