"""CPU-side checks of libkitgpu.so: it loads, exports every entry point of include/kitgpu.h,
and its host flattener validates topologies (no device needed for kg_topology_footprint)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from kitgpu import abi, cases
from kitgpu import build as B
from kitgpu import solver as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    B.build()
    return S.load_library()


def test_exports_every_declared_symbol(lib):
    hdr = open(os.path.join(ROOT, "include", "kitgpu.h")).read()
    declared = set(re.findall(r"^int\s+(kg_\w+)\s*\(", hdr, re.M))
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), name
    assert set(S.EXPORTS) <= declared


def test_footprint_without_device(lib):
    p = cases.sod(scale=0.125, nv=16)
    topo, _ = cases.build(p)
    b = S.topology_footprint(abi.make_params(p), topo)
    nf = int(np.diff(topo["grid_off"])[topo["cell_grid"]].sum()) * 2
    assert b >= nf * 8 * 4  # two f buffers and a dim-wide sdf at least


def test_rejects_inconsistent_topology(lib):
    p = cases.sod(scale=0.125, nv=16)
    topo, _ = cases.build(p)
    bad = dict(topo)
    bad["face_here"] = topo["face_here"].copy()
    bad["face_here"][0] = topo["n_cells"] + 5
    with pytest.raises(S.KitGpuError) as e:
        S.topology_footprint(abi.make_params(p), bad)
    assert e.value.code == 2


def test_rejects_zero_velocity_midpoint(lib):
    p = cases.couette(n=4, nv=8)
    topo, _ = cases.build(p)
    bad = dict(topo)
    bad["vs_midpoint"] = topo["vs_midpoint"].copy()
    bad["vs_midpoint"][3] = 0.0
    with pytest.raises(S.KitGpuError):
        S.topology_footprint(abi.make_params(p), bad)


def test_rejects_dvm_maxwell_domain(lib):
    p = cases.couette(n=4, nv=8)
    topo, _ = cases.build(p)
    with pytest.raises(S.KitGpuError) as e:
        S.topology_footprint(abi.make_params(p, flux=abi.KG_FLUX_DVM), topo)
    assert "undefined" in str(e.value)


def test_create_fails_loudly_without_device(lib):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a device is present")
    h = C.c_void_p()
    prm = abi.make_params(cases.couette(n=4, nv=8))
    rc = lib.kg_create(C.byref(prm), 0, C.byref(h))
    assert rc == 3  # KG_ERR_CUDA: no CPU fallback
