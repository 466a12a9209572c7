"""ctypes front end of the FP64 CPU oracle (oracle/kg_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py for the CPU baseline.  The product path never uses it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libkgoracle.so")
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "kitamr.jl_gb300"))
from kitgpu import abi  # noqa: E402

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "kg_oracle.cpp")):
            build()
        L = C.CDLL(LIB)
        L.kgo_sizes.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 4
        L.kgo_run.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int64, C.c_int32] + \
            [C.POINTER(C.c_double)] * 7 + [C.POINTER(C.c_double), C.POINTER(C.c_double),
                                           C.POINTER(C.c_int32), C.c_int32]
        L.kgo_moments.argtypes = [C.c_void_p, C.c_void_p] + [C.POINTER(C.c_double)] * 4
        L.kgo_macro_slope.argtypes = [C.c_void_p, C.c_void_p] + [C.POINTER(C.c_double)] * 2
        L.kgo_adapt.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p] + [C.POINTER(C.c_double)] * 10
        L.kgo_vs_flags.argtypes = [C.c_void_p, C.c_void_p] + [C.POINTER(C.c_double)] * 4 + \
            [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.kgo_slope.argtypes = [C.c_void_p, C.c_void_p] + [C.POINTER(C.c_double)] * 3 + [C.c_int32]
        L.kgo_criterion.argtypes = [C.c_void_p, C.c_void_p] + [C.POINTER(C.c_double)] * 3 + \
            [C.c_double, C.POINTER(C.c_double)]
        L.kgo_last_error.argtypes = [C.c_char_p, C.c_size_t]
        L.kgo_solution.argtypes = [C.c_void_p, C.c_void_p] + [C.POINTER(C.c_double)] * 7 + [C.c_int32]
        L.kgo_iprojection.argtypes = [C.c_int, C.c_int, C.c_int] + [C.POINTER(C.c_double)] * 5
        _lib = L
    return _lib


class OracleState:
    """Full state of one problem as the oracle advances it (cells and wall records)."""

    def __init__(self, topo: Dict, state: Dict):
        self.topo = topo
        self.tref = abi.TopologyRef(topo)
        n = [C.c_int64() for _ in range(4)]
        lib().kgo_sizes(C.cast(self.tref.ptr, C.c_void_p), *[C.byref(x) for x in n])
        nf, nsdf, nwf, nwsdf = [x.value for x in n]
        self.f = np.ascontiguousarray(state["f"], dtype=np.float64).copy()
        assert self.f.size == nf, (self.f.size, nf)
        self.sdf = np.zeros(max(nsdf, 1))
        self.w = np.ascontiguousarray(state["w"], dtype=np.float64).copy()
        self.prim = np.ascontiguousarray(state["prim"], dtype=np.float64).copy()
        dim = topo["dim"]
        self.qf = np.zeros(max(topo["n_cells"] * dim, 1))
        # SolidNeighbor df starts as a copy of the donor's df (Immersed_boundary.jl:290-298)
        self.wall_f = np.zeros(max(nwf, 1))
        self.wall_sdf = np.zeros(max(nwsdf, 1))
        if topo["n_walls"]:
            from kitgpu.mesh import f_offsets
            off = f_offsets(topo)
            pos = 0
            for wd in topo["wall_donor"]:
                blk = self.f[off[wd]:off[wd + 1]]
                self.wall_f[pos:pos + blk.size] = blk
                pos += blk.size
        self.sum_res = np.zeros(5)
        self.sum_avg = np.zeros(5)
        self.checked = C.c_int32(0)

    def run(self, params, dt: float, step0: int, nsteps: int, nthreads: int = 1):
        rc = lib().kgo_run(C.byref(params), C.cast(self.tref.ptr, C.c_void_p), dt, step0, nsteps,
                           abi.dptr(self.f), abi.dptr(self.sdf), abi.dptr(self.w), abi.dptr(self.prim),
                           abi.dptr(self.qf), abi.dptr(self.wall_f), abi.dptr(self.wall_sdf),
                           abi.dptr(self.sum_res), abi.dptr(self.sum_avg), C.byref(self.checked), nthreads)
        if rc != 0:
            buf = C.create_string_buffer(512)
            lib().kgo_last_error(buf, 512)
            raise RuntimeError(f"oracle failed: {abi.ERRORS.get(rc, rc)}: {buf.value.decode()}")
        return self

    def macro_slope(self, params):
        """sw of every cell (update_macro_slope!), shape (n_cells, dim, dim + 2)."""
        nc, dim = self.topo["n_cells"], self.topo["dim"]
        sw = np.zeros(nc * dim * (dim + 2))
        rc = lib().kgo_macro_slope(C.byref(params), C.cast(self.tref.ptr, C.c_void_p), abi.dptr(self.sdf), abi.dptr(sw))
        if rc != 0:
            raise RuntimeError(f"oracle macro_slope failed: {rc}")
        return sw.reshape(nc, dim, dim + 2)

    def slope(self, params, nthreads: int = 1):
        """slope! on the state as it stands (overwrites self.sdf)."""
        rc = lib().kgo_slope(C.byref(params), C.cast(self.tref.ptr, C.c_void_p), abi.dptr(self.f),
                             abi.dptr(self.sdf), abi.dptr(self.wall_f), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle slope failed: {rc}")
        return self

    def criterion(self, params, adapt_coeffi_ps, sw=None):
        """PsData.lohner of every cell (update_criterion! + buffer layer) from this state's
        w, prim and sw, shape (n_cells, dim, dim + 2).  Without sw it follows
        ps_adaptive_mesh_refinement! (Physical_space/AMR.jl:1108-1116): slope! on the current
        f, then the criterion on the macro slopes of those slopes."""
        nc, dim = self.topo["n_cells"], self.topo["dim"]
        if sw is None:
            self.slope(params)
            sw = self.macro_slope(params)
        sw = np.ascontiguousarray(sw, dtype=np.float64).reshape(-1)
        lo = np.zeros(nc * dim * (dim + 2))
        rc = lib().kgo_criterion(C.byref(params), C.cast(self.tref.ptr, C.c_void_p), abi.dptr(self.w),
                                 abi.dptr(self.prim), abi.dptr(sw), float(adapt_coeffi_ps), abi.dptr(lo))
        if rc != 0:
            raise RuntimeError(f"oracle criterion failed: {rc}")
        return lo.reshape(nc, dim, dim + 2)

    def adapt(self, params, topo_new: Dict, src: np.ndarray) -> "OracleState":
        """The state on the adapted mesh topo_new (ps_replace!): slope! on the current f, then
        per new cell the move src says (a kg_adapt_src record array, abi.ADAPT_SRC).  Returns
        a new OracleState whose walls start from their donors' f (amr_recover!)."""
        self.slope(params)
        src = np.ascontiguousarray(src, dtype=abi.ADAPT_SRC)
        assert src.size == topo_new["n_cells"]
        tnew = abi.TopologyRef(topo_new)
        n = [C.c_int64() for _ in range(4)]
        lib().kgo_sizes(C.cast(tnew.ptr, C.c_void_p), *[C.byref(x) for x in n])
        nf, nsdf = n[0].value, n[1].value
        nc, dim = topo_new["n_cells"], topo_new["dim"]
        f = np.zeros(max(nf, 1)); sdf = np.zeros(max(nsdf, 1))
        w = np.zeros(nc * (dim + 2)); prim = np.zeros(nc * (dim + 2)); qf = np.zeros(max(nc * dim, 1))
        rc = lib().kgo_adapt(C.byref(params), C.cast(self.tref.ptr, C.c_void_p), C.cast(tnew.ptr, C.c_void_p),
                             C.c_void_p(src.ctypes.data), abi.dptr(self.f), abi.dptr(self.sdf), abi.dptr(self.w),
                             abi.dptr(self.prim), abi.dptr(self.qf), abi.dptr(f), abi.dptr(sdf), abi.dptr(w),
                             abi.dptr(prim), abi.dptr(qf))
        if rc != 0:
            buf = C.create_string_buffer(512)
            lib().kgo_last_error(buf, 512)
            raise RuntimeError(f"oracle adapt failed: {abi.ERRORS.get(rc, rc)}: {buf.value.decode()}")
        out = OracleState(topo_new, dict(f=f[:nf], w=w, prim=prim))
        out.sdf[:] = sdf
        out.qf[:] = qf
        return out

    def vs_flags(self, params, vs_cfg):
        """vs_refine! / vs_coarsen!'s per-velocity flags on this state (bit 0 refine, bit 1
        coarsen on the current grid), the Löhner indicator and the Velocity_Resolution."""
        from kitgpu.mesh import f_offsets
        nv_total = int(f_offsets(self.topo)[-1]) // int(self.topo["ndf"])
        flags = np.zeros(max(nv_total, 1), np.uint8)
        eta = np.zeros(max(nv_total, 1))
        vr = np.zeros(2)
        rc = lib().kgo_vs_flags(C.byref(params), C.cast(self.tref.ptr, C.c_void_p), abi.dptr(self.f),
                                abi.dptr(self.sdf), abi.dptr(self.w), abi.dptr(self.prim), C.byref(vs_cfg),
                                C.c_void_p(flags.ctypes.data), C.c_void_p(eta.ctypes.data), C.c_void_p(vr.ctypes.data))
        if rc != 0:
            raise RuntimeError(f"oracle vs_flags failed: {rc}")
        return flags[:nv_total], eta[:nv_total], vr

    def solution(self, params, quad_index=None, n_quads=None, nthreads: int = 1):
        """save_result's rows on this state (changing it as save_result does: fresh slopes,
        updated solid cells, refreshed wall-direction slopes of the SolidNeighbors):
        PS_Solution prim / qf per quadrant (NaN rows for solid cells and quadrants without a
        cell) and per SolidNeighbor prim, qf and the pressure tensor."""
        nc, dim = self.topo["n_cells"], self.topo["dim"]
        nwall = int(self.topo["n_walls"])
        wr = 2 * dim + 2 + dim * (dim + 1) // 2
        rows = np.zeros(max(nwall, 1) * wr)
        rc = lib().kgo_solution(C.byref(params), C.cast(self.tref.ptr, C.c_void_p), abi.dptr(self.f),
                                abi.dptr(self.sdf), abi.dptr(self.w), abi.dptr(self.prim), abi.dptr(self.wall_f),
                                abi.dptr(self.wall_sdf), abi.dptr(rows), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle solution failed: {rc}")
        nq = nc if n_quads is None else int(n_quads)
        qi = np.arange(nc) if quad_index is None else np.asarray(quad_index)
        prim = np.full((nq, dim + 2), np.nan)
        qf = np.full((nq, dim), np.nan)
        be = np.asarray(self.topo["cell_bound_enc"])
        fl = be >= 0
        prim[qi[fl]] = self.prim.reshape(nc, dim + 2)[fl]
        qf[qi[fl]] = self.qf[:nc * dim].reshape(nc, dim)[fl]
        return {"prim": prim, "qf": qf, "walls": rows[:nwall * wr].reshape(nwall, wr)}

    def moments(self, params):
        nc, nw = self.topo["n_cells"], self.topo["dim"] + 2
        w = np.zeros(nc * nw)
        q = np.zeros(nc * self.topo["dim"])
        lib().kgo_moments(C.byref(params), C.cast(self.tref.ptr, C.c_void_p), abi.dptr(self.f),
                          abi.dptr(self.prim), abi.dptr(w), abi.dptr(q))
        return w.reshape(nc, nw), q.reshape(nc, self.topo["dim"])


def iprojection(dim: int, ndf: int, mid: np.ndarray, weight: np.ndarray, df: np.ndarray, w: np.ndarray):
    """conserved_I_porjection! of one velocity grid (Theory/I-projection.jl:144-158).

    mid: nv x dim midpoints, weight: nv, df: nv x ndf, w: dim+2 conserved variables.
    Returns the projected df (nv x ndf) and the multipliers λ (dim+2)."""
    nv = weight.size
    m = np.ascontiguousarray(np.asarray(mid, np.float64).reshape(nv, dim).T).ravel()
    wt = np.ascontiguousarray(weight, np.float64)
    f = np.ascontiguousarray(np.asarray(df, np.float64).reshape(nv, ndf).T).ravel()
    ww = np.ascontiguousarray(w, np.float64)
    lam = np.zeros(dim + 2)
    rc = lib().kgo_iprojection(dim, ndf, nv, abi.dptr(m), abi.dptr(wt), abi.dptr(f), abi.dptr(ww), abi.dptr(lam))
    if rc != 0:
        raise RuntimeError(f"oracle iprojection failed: {rc}")
    return f.reshape(ndf, nv).T.copy(), lam
