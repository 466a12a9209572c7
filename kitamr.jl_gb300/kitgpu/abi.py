"""ctypes mirror of include/kitgpu.h: the parameter, topology and report structs, and the
marshalling of a topology dict (numpy arrays) into a ``kg_topology``."""
from __future__ import annotations

import ctypes as C
from typing import Dict

import numpy as np

KG_OK = 0
KG_FLUX_CAIDVM, KG_FLUX_DVM = 0, 1
KG_MARCH_CAIDVM, KG_MARCH_EULER, KG_MARCH_CIP = 0, 1, 2
KG_PREC_FP64, KG_PREC_MIXED = 0, 1

ERRORS = {
    0: "KG_OK", 1: "KG_ERR_ARG", 2: "KG_ERR_TOPOLOGY", 3: "KG_ERR_CUDA", 4: "KG_ERR_NOMEM",
    5: "KG_ERR_NONFINITE", 6: "KG_ERR_NEGATIVE", 7: "KG_ERR_STATE", 8: "KG_ERR_BUDGET",
    9: "KG_ERR_TIMEOUT",
}

_p = C.c_void_p


class KgParams(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("ndf", C.c_int32), ("flux", C.c_int32), ("marching", C.c_int32),
        ("precision", C.c_int32), ("st_check_interval", C.c_int32),
        ("gamma", C.c_double), ("K", C.c_double), ("Pr", C.c_double), ("omega", C.c_double),
        ("mu_ref", C.c_double),
    ]


_TOPO_FIELDS = [
    ("dim", C.c_int32), ("ndf", C.c_int32),
    ("n_grids", C.c_int32), ("grid_off", _p), ("vs_level", _p), ("vs_weight", _p), ("vs_midpoint", _p),
    ("n_cells", C.c_int32), ("cell_bound_enc", _p), ("cell_level", _p), ("cell_grid", _p),
    ("cell_midpoint", _p), ("cell_ds", _p),
    ("nbr_state", _p), ("nbr_off", _p), ("nbr_ref", _p),
    ("n_walls", C.c_int32), ("wall_donor", _p), ("wall_solid", _p), ("wall_faceid", _p),
    ("wall_aux_point", _p), ("wall_normal", _p), ("wall_bc", _p), ("wall_cut_off", _p),
    ("wall_cut_index", _p), ("wall_cut_gas_w", _p), ("wall_cut_solid_w", _p),
    ("n_faces", C.c_int32), ("face_kind", _p), ("face_dir", _p), ("face_rot", _p), ("face_area", _p),
    ("face_midpoint", _p), ("face_here", _p), ("face_there", _p), ("face_there_midpoint", _p),
    ("face_bc_kind", _p), ("face_bc", _p),
]

_DTYPES = {
    "grid_off": np.int64, "vs_level": np.int8, "vs_weight": np.float64, "vs_midpoint": np.float64,
    "cell_bound_enc": np.int32, "cell_level": np.int32, "cell_grid": np.int32,
    "cell_midpoint": np.float64, "cell_ds": np.float64,
    "nbr_state": np.int8, "nbr_off": np.int32, "nbr_ref": np.int32,
    "wall_donor": np.int32, "wall_solid": np.int32, "wall_faceid": np.int32,
    "wall_aux_point": np.float64, "wall_normal": np.float64, "wall_bc": np.float64,
    "wall_cut_off": np.int32, "wall_cut_index": np.int32, "wall_cut_gas_w": np.float64,
    "wall_cut_solid_w": np.float64,
    "face_kind": np.int8, "face_dir": np.int8, "face_rot": np.float64, "face_area": np.float64,
    "face_midpoint": np.float64, "face_here": np.int32, "face_there": np.int32,
    "face_there_midpoint": np.float64, "face_bc_kind": np.int8, "face_bc": np.float64,
}


class KgTopology(C.Structure):
    _fields_ = _TOPO_FIELDS


class KgStepReport(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("checked", C.c_int32), ("checked_step", C.c_int64),
        ("sum_res", C.c_double * 5), ("sum_avg", C.c_double * 5), ("device_ms", C.c_double),
        ("phase_cells", C.c_int64), ("kernel_launches", C.c_int32),
    ]


class TopologyRef:
    """A ``kg_topology`` plus the contiguous numpy arrays it points into (kept alive)."""

    def __init__(self, topo: Dict):
        self.arrays = {}
        self.struct = KgTopology()
        for name, ctype in _TOPO_FIELDS:
            if ctype is _p:
                arr = np.ascontiguousarray(np.asarray(topo[name], dtype=_DTYPES[name]))
                if arr.size == 0:
                    arr = np.zeros(1, dtype=_DTYPES[name])  # a valid pointer for empty arrays
                self.arrays[name] = arr
                setattr(self.struct, name, arr.ctypes.data)
            else:
                setattr(self.struct, name, int(topo[name]))

    @property
    def ptr(self):
        return C.byref(self.struct)


def make_params(problem, precision=KG_PREC_FP64, flux=KG_FLUX_CAIDVM, marching=KG_MARCH_CAIDVM,
                st_check_interval=100) -> KgParams:
    g = problem.gas
    dim = problem.case.dim
    return KgParams(dim=dim, ndf=2 if dim == 2 else 1, flux=flux, marching=marching,
                    precision=precision, st_check_interval=st_check_interval,
                    gamma=g.gamma, K=g.K, Pr=g.Pr, omega=g.omega, mu_ref=g.mu_ref())


KG_ADAPT_KEEP, KG_ADAPT_REFINE, KG_ADAPT_COARSEN, KG_ADAPT_VS = 0, 1, 2, 3
KG_ADAPT_MAX_DEPTH = 8
# kg_adapt_src: where a cell of an adapted mesh takes its state from
ADAPT_SRC = np.dtype([("kind", "<i4"), ("depth", "<i4"), ("src", "<i4", (8,)), ("path", "i1", (KG_ADAPT_MAX_DEPTH,))])
assert ADAPT_SRC.itemsize == 48


KG_VS_LOHNER, KG_VS_CONTRIBUTION = 0, 1


class KgVsConfig(C.Structure):
    _fields_ = [
        ("quadrature", C.c_double * 6), ("vs_trees_num", C.c_int32 * 3), ("maxlevel", C.c_int32),
        ("mode", C.c_int32), ("pad", C.c_int32), ("coeffi_lohner", C.c_double), ("coeffi_local", C.c_double),
        ("coeffi_global", C.c_double),
    ]


def make_vs_config(problem, maxlevel=None, mode=KG_VS_LOHNER, coeffi_lohner=0.6, coeffi_local=1e-2,
                   coeffi_global=0.125) -> KgVsConfig:
    """The velocity-space adaptation settings of a case (solver defaults of Solver/Types.jl:97-100)."""
    c = problem.case
    q = list(c.quadrature) + [0.0] * (6 - len(c.quadrature))
    tn = list(c.vs_trees_num) + [1] * (3 - len(c.vs_trees_num))
    ml = problem.vs_maxlevel if maxlevel is None else maxlevel
    return KgVsConfig(quadrature=(C.c_double * 6)(*q), vs_trees_num=(C.c_int32 * 3)(*tn), maxlevel=ml, mode=mode,
                      pad=0, coeffi_lohner=coeffi_lohner, coeffi_local=coeffi_local, coeffi_global=coeffi_global)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))
