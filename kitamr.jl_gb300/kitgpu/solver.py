"""Python host mirror of the GPU step: ctypes binding of libkitgpu.so.

The reference advances a step with ``slope!(p4est, ka); flux!(p4est, ka); iterate!(p4est, ka)``
(src/Solver/Solver.jl:65-67).  ``GpuStep.step`` is that triple on the device; the state
moves to and from the host only through ``upload_state`` / ``download_state`` (the sync
points around adaptation, output and restart).  There is no CPU fallback: loading fails
with an exception when the library or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Optional

import numpy as np

from . import abi
from .build import LIB

_lib = None


def load_library(path: Optional[str] = None):
    global _lib
    if _lib is not None:
        return _lib
    p = path or os.environ.get("KITGPU_LIB", LIB)
    if not os.path.exists(p):
        raise RuntimeError(f"libkitgpu.so not built ({p}); run kitgpu/build.py or __graft_entry__.build()")
    L = C.CDLL(p)
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    L.kg_create.argtypes = [vp, C.c_int, C.POINTER(vp)]
    L.kg_destroy.argtypes = [vp]
    L.kg_upload_topology.argtypes = [vp, vp]
    L.kg_upload_state.argtypes = [vp, vp, vp, vp]
    L.kg_download_state.argtypes = [vp, vp, vp, vp, vp, vp]
    L.kg_step.argtypes = [vp, dbl, i64, i32, vp]
    L.kg_profile_enable.argtypes = [vp, C.c_int]
    L.kg_profile_read.argtypes = [vp, C.POINTER(C.c_char_p), C.POINTER(dbl), C.POINTER(i64), i32, C.POINTER(i32)]
    L.kg_profile_units.argtypes = [vp, C.POINTER(i64), i32, C.POINTER(i32)]
    L.kg_memory_footprint.argtypes = [vp, C.POINTER(i64)]
    L.kg_topology_footprint.argtypes = [vp, vp, C.POINTER(i64)]
    L.kg_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.kg_use_graph.argtypes = [vp, C.c_int]
    L.kg_device_flatten.argtypes = [vp, C.c_int]
    L.kg_layout_read.argtypes = [vp, C.c_char_p, vp, i64, C.POINTER(i64)]
    L.kg_batch_create.argtypes = [vp, C.c_int, i64, C.POINTER(vp)]
    L.kg_batch_admit.argtypes = [vp, vp, vp, vp, vp, vp, dbl, i64, C.POINTER(i32)]
    L.kg_batch_release.argtypes = [vp, i32]
    L.kg_batch_step.argtypes = [vp, i32, vp, i32]
    L.kg_batch_download.argtypes = [vp, i32, vp, vp, vp, vp]
    L.kg_batch_info.argtypes = [vp, C.POINTER(i32), C.POINTER(i64), C.POINTER(i64)]
    L.kg_batch_set_dt.argtypes = [vp, i32, dbl]
    L.kg_autotune.argtypes = [vp, C.c_int]
    L.kg_fuse_slopes.argtypes = [vp, C.c_int]
    L.kg_download_sw.argtypes = [vp, vp]
    L.kg_batch_download_sw.argtypes = [vp, i32, vp]
    L.kg_criterion.argtypes = [vp, dbl, vp]
    L.kg_batch_criterion.argtypes = [vp, i32, dbl, vp]
    L.kg_adapt.argtypes = [vp, vp, vp]
    L.kg_batch_adapt.argtypes = [vp, i32, vp, vp]
    L.kg_download_restart.argtypes = [vp, vp, i32, vp, vp]
    L.kg_vs_flags.argtypes = [vp, vp, vp, vp, vp]
    L.kg_batch_vs_flags.argtypes = [vp, i32, vp, vp, vp, vp]
    L.kg_upload_restart.argtypes = [vp, vp, i32, vp, vp]
    L.kg_download_solution.argtypes = [vp, vp, i32, vp, vp, vp]
    L.kg_batch_download_restart.argtypes = [vp, i32, vp, i32, vp, vp]
    L.kg_autotune_result.argtypes = [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(dbl), i32]
    L.kg_serve.argtypes = [vp, i32, vp, vp, vp, dbl, i64, i32, vp, vp, vp, vp, vp]
    L.kg_vs_conserve.argtypes = [vp, vp]
    L.kg_batch_vs_conserve.argtypes = [vp, i32, vp]
    _lib = L
    return L


def _profile_read(L, h):
    cap = 32
    names = (C.c_char_p * cap)()
    ms = (C.c_double * cap)()
    cnt = (C.c_int64 * cap)()
    units = (C.c_int64 * cap)()
    n = C.c_int32()
    _check(L, h, L.kg_profile_read(h, names, ms, cnt, cap, C.byref(n)))
    m = C.c_int32()
    _check(L, h, L.kg_profile_units(h, units, cap, C.byref(m)))
    return {names[i].decode(): (ms[i], cnt[i], units[i]) for i in range(min(n.value, cap))}


EXPORTS = [
    "kg_create", "kg_destroy", "kg_upload_topology", "kg_upload_state", "kg_download_state",
    "kg_step", "kg_profile_enable", "kg_profile_read", "kg_profile_units", "kg_memory_footprint",
    "kg_topology_footprint", "kg_last_error", "kg_use_graph",
    "kg_batch_create", "kg_batch_admit", "kg_batch_release", "kg_batch_step", "kg_batch_download",
    "kg_batch_info", "kg_batch_set_dt", "kg_autotune", "kg_autotune_result", "kg_fuse_slopes",
    "kg_download_sw", "kg_batch_download_sw", "kg_criterion", "kg_batch_criterion",
    "kg_adapt", "kg_batch_adapt", "kg_download_restart", "kg_upload_restart", "kg_batch_download_restart",
    "kg_download_solution",
    "kg_vs_flags", "kg_batch_vs_flags", "kg_serve", "kg_vs_conserve", "kg_batch_vs_conserve",
]


def _autotune_result(L, h):
    sch, ctas = C.c_int32(), C.c_int32()
    ms = (C.c_double * 8)()
    _check(L, h, L.kg_autotune_result(h, C.byref(sch), C.byref(ctas), ms, 8))
    return {"schedule": sch.value, "ctas_per_sm": ctas.value, "trial_ms": [ms[i] for i in range(8) if ms[i] > 0]}


class KitGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{abi.ERRORS.get(code, code)}: {msg}")
        self.code = code


def _check(L, h, rc):
    if rc != 0:
        buf = C.create_string_buffer(1024)
        L.kg_last_error(h, buf, 1024)
        raise KitGpuError(rc, buf.value.decode(errors="replace"))


def topology_footprint(params: abi.KgParams, topo: Dict) -> int:
    L = load_library()
    tref = abi.TopologyRef(topo)
    b = C.c_int64()
    _check(L, None, L.kg_topology_footprint(C.byref(params), C.cast(tref.ptr, C.c_void_p), C.byref(b)))
    return b.value


class GpuStep:
    """One libkitgpu handle holding one topology and its state on one device."""

    def __init__(self, params: abi.KgParams, topo: Dict, device: int = 0, device_flatten: bool = True):
        self.L = load_library()
        self.params = params
        self.topo = topo
        h = C.c_void_p()
        _check(self.L, None, self.L.kg_create(C.byref(params), device, C.byref(h)))
        self.h = h
        # the gather form of the topology built on the device (default) or on the host
        _check(self.L, self.h, self.L.kg_device_flatten(self.h, int(device_flatten)))
        self._tref = abi.TopologyRef(topo)
        _check(self.L, self.h, self.L.kg_upload_topology(self.h, C.cast(self._tref.ptr, C.c_void_p)))
        from .mesh import f_offsets
        self.foff = f_offsets(topo)
        self.nc = int(topo["n_cells"])
        self.dim = int(topo["dim"])

    def close(self):
        if self.h:
            self.L.kg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_state(self, f: np.ndarray, w: np.ndarray, prim: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        assert f.size == self.foff[-1] and w.size == self.nc * (self.dim + 2)
        _check(self.L, self.h, self.L.kg_upload_state(self.h, f.ctypes.data, w.ctypes.data, prim.ctypes.data))

    def step(self, dt: float, step0: int, nsteps: int) -> abi.KgStepReport:
        rep = abi.KgStepReport()
        _check(self.L, self.h, self.L.kg_step(self.h, dt, step0, nsteps, C.byref(rep)))
        return rep

    def serve(self, states, dt: float, step0: int, nsteps: int, outputs=None):
        """kg_serve: every state dict (f, w, prim: float64 arrays, pinned for overlapped copies)
        is advanced nsteps steps from step0; returns (outputs, reports).  `outputs`: optional
        list of dicts of preallocated f, w, prim, qf arrays (entries may be shared between
        requests)."""
        n = len(states)
        nf, nw = int(self.foff[-1]), self.nc * (self.dim + 2)
        ins = [{k: np.ascontiguousarray(st[k], dtype=np.float64) for k in ("f", "w", "prim")} for st in states]
        for st in ins:
            assert st["f"].size == nf and st["w"].size == nw and st["prim"].size == nw
        if outputs is None:
            outputs = [dict(f=np.empty(nf), w=np.empty(nw), prim=np.empty(nw), qf=np.empty(self.nc * self.dim))
                       for _ in range(n)]
        ptrs = lambda key, lst: (C.c_void_p * n)(*[a[key].ctypes.data if a.get(key) is not None else None for a in lst])
        reports = (abi.KgStepReport * max(n, 1))()
        _check(self.L, self.h, self.L.kg_serve(self.h, n, ptrs("f", ins), ptrs("w", ins), ptrs("prim", ins), dt, step0,
                                               nsteps, ptrs("f", outputs), ptrs("w", outputs), ptrs("prim", outputs),
                                               ptrs("qf", outputs), reports))
        return outputs, [reports[r] for r in range(n)]

    def vs_conserve(self, cell_flags: np.ndarray):
        """kg_vs_conserve: I-projection of the flagged cells' f onto their w (in place on the device)."""
        fl = np.ascontiguousarray(cell_flags, dtype=np.uint8)
        assert fl.size == self.nc
        _check(self.L, self.h, self.L.kg_vs_conserve(self.h, fl.ctypes.data))

    def download_state(self, sdf: bool = False, f: bool = True) -> Dict[str, np.ndarray]:
        """f (unless f=False), w, prim, qf and optionally sdf of every cell."""
        nf = int(self.foff[-1])
        out = dict(w=np.empty(self.nc * (self.dim + 2)), prim=np.empty(self.nc * (self.dim + 2)),
                   qf=np.empty(self.nc * self.dim))
        if f:
            out["f"] = np.empty(nf)
        if sdf:
            out["sdf"] = np.empty(nf * self.dim)
        _check(self.L, self.h, self.L.kg_download_state(
            self.h, out["f"].ctypes.data if f else None, out["w"].ctypes.data, out["prim"].ctypes.data,
            out["qf"].ctypes.data, out["sdf"].ctypes.data if sdf else None))
        return out

    def download_sw(self) -> np.ndarray:
        """sw of every cell (update_macro_slope!), shape (n_cells, dim, dim + 2)."""
        sw = np.empty(self.nc * self.dim * (self.dim + 2))
        _check(self.L, self.h, self.L.kg_download_sw(self.h, sw.ctypes.data))
        return sw.reshape(self.nc, self.dim, self.dim + 2)

    def criterion(self, adapt_coeffi_ps: float) -> np.ndarray:
        """PsData.lohner of every cell (update_criterion! + buffer layer), shape (n_cells, dim, dim + 2)."""
        lo = np.empty(self.nc * self.dim * (self.dim + 2))
        _check(self.L, self.h, self.L.kg_criterion(self.h, float(adapt_coeffi_ps), lo.ctypes.data))
        return lo.reshape(self.nc, self.dim, self.dim + 2)

    def adapt(self, topo: Dict, src: np.ndarray):
        """Move the device state onto the adapted mesh ``topo`` (kg_adapt); ``src`` holds one
        abi.ADAPT_SRC record per cell of ``topo``.  A rejected plan leaves the handle as it was."""
        tref = abi.TopologyRef(topo)
        src = np.ascontiguousarray(src, dtype=abi.ADAPT_SRC)
        if src.size != int(topo["n_cells"]):
            raise ValueError("one adaptation record per cell of the new topology")
        _check(self.L, self.h, self.L.kg_adapt(self.h, C.cast(tref.ptr, C.c_void_p), src.ctypes.data))
        from .mesh import f_offsets
        self.topo, self._tref = topo, tref
        self.foff = f_offsets(topo)
        self.nc = int(topo["n_cells"])

    def vs_flags(self, vs_cfg: abi.KgVsConfig, eta: bool = True):
        """vs_refine! / vs_coarsen!'s per-velocity flags (bit 0 refine, bit 1 coarsen on the
        current grid), the Löhner indicator (or None) and the Velocity_Resolution."""
        nv_total = int(self.foff[self.nc]) // int(self.topo["ndf"])
        fl = np.empty(max(nv_total, 1), np.uint8)
        et = np.empty(max(nv_total, 1)) if eta else None
        vr = np.empty(2)
        _check(self.L, self.h, self.L.kg_vs_flags(self.h, C.byref(vs_cfg), fl.ctypes.data,
                                                    et.ctypes.data if eta else None, vr.ctypes.data))
        return fl[:nv_total], (et[:nv_total] if eta else None), vr

    def download_restart(self, quad_index: Optional[np.ndarray] = None, n_quads: Optional[int] = None):
        """The state arrays of save_for_restart: vs_df (Nv x ndf) and ws (n_quads x dim+2)."""
        ndf = int(self.topo["ndf"])
        nq = self.nc if n_quads is None else int(n_quads)
        qi = None if quad_index is None else np.ascontiguousarray(quad_index, dtype=np.int32)
        vs_df = np.empty(int(self.foff[self.nc]), dtype=np.float64)
        ws = np.empty(nq * (self.dim + 2))
        _check(self.L, self.h, self.L.kg_download_restart(self.h, None if qi is None else qi.ctypes.data, nq,
                                                            vs_df.ctypes.data, ws.ctypes.data))
        return vs_df.reshape(ndf, -1).T, ws.reshape(self.dim + 2, nq).T

    def download_solution(self, quad_index: Optional[np.ndarray] = None, n_quads: Optional[int] = None):
        """save_result's rows (kg_download_solution): PS_Solution prim (n_quads, dim+2) and qf
        (n_quads, dim) with NaN rows for solid cells and quadrants without a cell, and per
        SolidNeighbor record prim, qf and the pressure tensor (n_walls, 2 dim + 2 + dim (dim+1)/2)."""
        nq = self.nc if n_quads is None else int(n_quads)
        qi = None if quad_index is None else np.ascontiguousarray(quad_index, dtype=np.int32)
        d = self.dim
        wr = 2 * d + 2 + d * (d + 1) // 2
        nwall = int(self.topo["n_walls"])
        prim = np.empty(nq * (d + 2))
        qf = np.empty(nq * d)
        walls = np.empty(max(nwall, 1) * wr)
        _check(self.L, self.h, self.L.kg_download_solution(self.h, None if qi is None else qi.ctypes.data, nq,
                                                             prim.ctypes.data, qf.ctypes.data, walls.ctypes.data))
        return {"prim": prim.reshape(nq, d + 2), "qf": qf.reshape(nq, d), "walls": walls[:nwall * wr].reshape(nwall, wr)}

    def upload_restart(self, vs_df: np.ndarray, ws: np.ndarray, quad_index: Optional[np.ndarray] = None):
        """restart(): f from vs_df, w from ws, prim = get_prim(w)."""
        vs = np.asfortranarray(vs_df, dtype=np.float64)
        wsf = np.asfortranarray(ws, dtype=np.float64)
        qi = None if quad_index is None else np.ascontiguousarray(quad_index, dtype=np.int32)
        _check(self.L, self.h, self.L.kg_upload_restart(self.h, None if qi is None else qi.ctypes.data,
                                                          int(wsf.shape[0]), vs.ctypes.data, wsf.ctypes.data))

    def profile(self, enable: bool = True):
        _check(self.L, self.h, self.L.kg_profile_enable(self.h, int(enable)))

    def autotune(self, enable: bool = True):
        _check(self.L, self.h, self.L.kg_autotune(self.h, int(enable)))

    def fuse_slopes(self, enable: bool = True):
        _check(self.L, self.h, self.L.kg_fuse_slopes(self.h, int(enable)))

    def device_flatten(self, enable: bool = True):
        """Builder of the gather form for later topology changes: device (True) or host."""
        _check(self.L, self.h, self.L.kg_device_flatten(self.h, int(enable)))

    def layout_read(self, name: str) -> bytes:
        """The named array of the gather form the next step reads, as raw bytes."""
        n = C.c_int64()
        _check(self.L, self.h, self.L.kg_layout_read(self.h, name.encode(), None, 0, C.byref(n)))
        buf = (C.c_char * max(n.value, 1))()
        _check(self.L, self.h, self.L.kg_layout_read(self.h, name.encode(), buf, n.value, C.byref(n)))
        return bytes(buf[: n.value])

    def autotune_result(self):
        return _autotune_result(self.L, self.h)

    def profile_read(self):
        """name -> (total ms, launches, phase cells processed) of the profiled launches."""
        return _profile_read(self.L, self.h)

    def use_graph(self, enable: bool = True):
        _check(self.L, self.h, self.L.kg_use_graph(self.h, int(enable)))

    def memory_footprint(self) -> int:
        b = C.c_int64()
        _check(self.L, self.h, self.L.kg_memory_footprint(self.h, C.byref(b)))
        return b.value


MAX_SLOTS = 4096


class GpuBatch:
    """A batch handle: independent problems advanced together on one device."""

    def __init__(self, params: abi.KgParams, pool_bytes: int, device: int = 0, device_flatten: bool = True):
        self.L = load_library()
        self.params = params
        h = C.c_void_p()
        _check(self.L, None, self.L.kg_batch_create(C.byref(params), device, int(pool_bytes), C.byref(h)))
        self.h = h
        # the gather form of admitted / adapted problems built on the device (default) or host
        _check(self.L, self.h, self.L.kg_device_flatten(self.h, int(device_flatten)))
        self.meta = {}            # slot -> (topo, foff)
        self._reports = (abi.KgStepReport * MAX_SLOTS)()

    def close(self):
        if self.h:
            self.L.kg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, params: abi.KgParams, topo: Dict, f, w, prim, dt: float, step: int = 0) -> int:
        """Admit a problem; raises KitGpuError with code KG_ERR_BUDGET (8) when it does not fit."""
        tref = abi.TopologyRef(topo)
        f = np.ascontiguousarray(f, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        slot = C.c_int32()
        _check(self.L, self.h, self.L.kg_batch_admit(self.h, C.byref(params), C.cast(tref.ptr, C.c_void_p),
                                                       f.ctypes.data, w.ctypes.data, prim.ctypes.data, dt, step,
                                                       C.byref(slot)))
        from .mesh import f_offsets
        self.meta[slot.value] = (topo, f_offsets(topo))
        return slot.value

    def release(self, slot: int):
        _check(self.L, self.h, self.L.kg_batch_release(self.h, slot))
        self.meta.pop(slot, None)

    def step(self, nsteps: int = 1) -> Dict[int, abi.KgStepReport]:
        _check(self.L, self.h, self.L.kg_batch_step(self.h, nsteps, self._reports, MAX_SLOTS))
        return {s: self._reports[s] for s in self.meta}

    def download(self, slot: int) -> Dict[str, np.ndarray]:
        topo, foff = self.meta[slot]
        nc, dim = int(topo["n_cells"]), int(topo["dim"])
        out = dict(f=np.empty(int(foff[-1])), w=np.empty(nc * (dim + 2)), prim=np.empty(nc * (dim + 2)),
                   qf=np.empty(nc * dim))
        _check(self.L, self.h, self.L.kg_batch_download(self.h, slot, out["f"].ctypes.data, out["w"].ctypes.data,
                                                          out["prim"].ctypes.data, out["qf"].ctypes.data))
        return out

    def download_sw(self, slot: int) -> np.ndarray:
        topo, _ = self.meta[slot]
        nc, dim = int(topo["n_cells"]), int(topo["dim"])
        sw = np.empty(nc * dim * (dim + 2))
        _check(self.L, self.h, self.L.kg_batch_download_sw(self.h, slot, sw.ctypes.data))
        return sw.reshape(nc, dim, dim + 2)

    def criterion(self, slot: int, adapt_coeffi_ps: float) -> np.ndarray:
        topo, _ = self.meta[slot]
        nc, dim = int(topo["n_cells"]), int(topo["dim"])
        lo = np.empty(nc * dim * (dim + 2))
        _check(self.L, self.h, self.L.kg_batch_criterion(self.h, slot, float(adapt_coeffi_ps), lo.ctypes.data))
        return lo.reshape(nc, dim, dim + 2)

    def adapt(self, slot: int, topo: Dict, src: np.ndarray):
        """kg_batch_adapt: move one problem's state onto its adapted mesh ``topo``."""
        tref = abi.TopologyRef(topo)
        src = np.ascontiguousarray(src, dtype=abi.ADAPT_SRC)
        if src.size != int(topo["n_cells"]):
            raise ValueError("one adaptation record per cell of the new topology")
        _check(self.L, self.h, self.L.kg_batch_adapt(self.h, slot, C.cast(tref.ptr, C.c_void_p), src.ctypes.data))
        from .mesh import f_offsets
        self.meta[slot] = (topo, f_offsets(topo))

    def vs_flags(self, slot: int, vs_cfg: abi.KgVsConfig, eta: bool = True):
        topo, foff = self.meta[slot]
        nv_total = int(foff[int(topo["n_cells"])]) // int(topo["ndf"])
        fl = np.empty(max(nv_total, 1), np.uint8)
        et = np.empty(max(nv_total, 1)) if eta else None
        vr = np.empty(2)
        _check(self.L, self.h, self.L.kg_batch_vs_flags(self.h, slot, C.byref(vs_cfg), fl.ctypes.data,
                                                          et.ctypes.data if eta else None, vr.ctypes.data))
        return fl[:nv_total], (et[:nv_total] if eta else None), vr

    def download_restart(self, slot: int, quad_index: Optional[np.ndarray] = None, n_quads: Optional[int] = None):
        topo, foff = self.meta[slot]
        nc, dim, ndf = int(topo["n_cells"]), int(topo["dim"]), int(topo["ndf"])
        nq = nc if n_quads is None else int(n_quads)
        qi = None if quad_index is None else np.ascontiguousarray(quad_index, dtype=np.int32)
        vs_df = np.empty(int(foff[nc]), dtype=np.float64)
        ws = np.empty(nq * (dim + 2))
        _check(self.L, self.h, self.L.kg_batch_download_restart(self.h, slot, None if qi is None else qi.ctypes.data,
                                                                  nq, vs_df.ctypes.data, ws.ctypes.data))
        return vs_df.reshape(ndf, -1).T, ws.reshape(dim + 2, nq).T

    def info(self):
        n, fr, bpe = C.c_int32(), C.c_int64(), C.c_int64()
        _check(self.L, self.h, self.L.kg_batch_info(self.h, C.byref(n), C.byref(fr), C.byref(bpe)))
        return n.value, fr.value * bpe.value

    def set_dt(self, slot: int, dt: float):
        _check(self.L, self.h, self.L.kg_batch_set_dt(self.h, slot, dt))

    def use_graph(self, enable: bool = True):
        _check(self.L, self.h, self.L.kg_use_graph(self.h, int(enable)))

    def profile(self, enable: bool = True):
        _check(self.L, self.h, self.L.kg_profile_enable(self.h, int(enable)))

    def profile_read(self):
        """name -> (total ms, launches, phase cells processed) of the profiled launches."""
        return _profile_read(self.L, self.h)

    def autotune(self, enable: bool = True):
        _check(self.L, self.h, self.L.kg_autotune(self.h, int(enable)))

    def fuse_slopes(self, enable: bool = True):
        _check(self.L, self.h, self.L.kg_fuse_slopes(self.h, int(enable)))

    def layout_read(self, name: str) -> bytes:
        """The named array of the merged gather form the next step reads, as raw bytes."""
        return GpuStep.layout_read(self, name)

    def autotune_result(self):
        return _autotune_result(self.L, self.h)
