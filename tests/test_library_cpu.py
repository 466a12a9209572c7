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


def test_accepts_cip_marching_with_immersed_boundaries(lib):
    # iterate!(CIP_Marching) calls positivity_preserving_ib! next to walls (built: the flux
    # kernel's CIP variant for layouts with walls); such meshes lay out like any other
    p = cases.cylinder(scale=0.25, nv=8, vs_levels=0)
    topo, _ = cases.build(p)
    assert topo["n_walls"] > 0
    assert S.topology_footprint(abi.make_params(p, marching=abi.KG_MARCH_CIP), topo) > 0


def test_create_fails_loudly_without_device(lib):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a device is present")
    h = C.c_void_p()
    prm = abi.make_params(cases.couette(n=4, nv=8))
    rc = lib.kg_create(C.byref(prm), 0, C.byref(h))
    assert rc == 3  # KG_ERR_CUDA: no CPU fallback


def test_create_rejects_bad_parameters_before_touching_a_device(lib):
    prm = abi.make_params(cases.couette(n=4, nv=8))
    h = C.c_void_p()
    for field, value in (("dim", 4), ("precision", 7), ("flux", 9), ("st_check_interval", 0)):
        bad = abi.KgParams.from_buffer_copy(prm)
        setattr(bad, field, value)
        assert lib.kg_create(C.byref(bad), 0, C.byref(h)) == 1, field   # KG_ERR_ARG
        buf = C.create_string_buffer(256)
        lib.kg_last_error(None, buf, 256)
        assert buf.value, field


@pytest.mark.parametrize("make", [lambda: cases.box3d(n=(4, 3, 3), nv=6, levels=1),
                                  lambda: cases.sphere(scale=0.2, nv=6)], ids=["box3d", "sphere"])
def test_flattens_3d_topologies(lib, make):
    p = make()
    topo, _ = cases.build(p)
    for prec in (abi.KG_PREC_FP64, abi.KG_PREC_MIXED):
        assert S.topology_footprint(abi.make_params(p, precision=prec), topo) > 0


def test_reference_arm_prints_the_contract_line():
    """bench.py --impl reference: the reference's CPU path (the oracle port) on the bench's
    workload, one JSON line with the keys of the benchmark contract."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "phase-cell updates/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def _footprint_error(p, topo, **prm):
    with pytest.raises(S.KitGpuError) as e:
        S.topology_footprint(abi.make_params(p, **prm), topo)
    return e.value


@pytest.mark.parametrize("mutate,code,words", [
    # a grid whose levels cannot tile the root lattice next to another grid (the merge walk)
    ("ragged_grid", 2, "tile"),
    # cell_grid out of range
    ("bad_cell_grid", 2, "cell_grid"),
    # an empty velocity grid
    ("empty_grid", 2, "empty"),
    # a face whose direction is not a dimension
    ("bad_face_dir", 2, "face_dir"),
    # an unknown domain boundary kind
    ("bad_bc_kind", 2, "boundary kind"),
    # no cells at all
    ("no_cells", 2, "empty"),
])
def test_flattener_rejects_malformed_topologies(lib, mutate, code, words):
    p = cases.collision(center=0.5)        # two velocity grids, hanging faces, outflow + periodic
    topo, _ = cases.build(p)
    bad = dict(topo)
    if mutate == "ragged_grid":
        # drop the last velocity cell of grid 1: its leaves no longer cover the root lattice
        goff = np.asarray(topo["grid_off"]).copy()
        cut = int(goff[2]) - 1
        keep = np.ones(int(goff[-1]), bool)
        keep[cut] = False
        bad["vs_level"] = np.asarray(topo["vs_level"])[keep]
        bad["vs_weight"] = np.asarray(topo["vs_weight"])[keep]
        mid = np.asarray(topo["vs_midpoint"])
        parts = []
        for g in range(int(topo["n_grids"])):
            a, b = int(goff[g]), int(goff[g + 1])
            blk = mid[a * 2:b * 2].reshape(2, b - a)
            if g == 1:
                blk = blk[:, :-1]
            parts.append(blk.reshape(-1))
        bad["vs_midpoint"] = np.concatenate(parts)
        goff[2:] -= 1
        bad["grid_off"] = goff
    elif mutate == "bad_cell_grid":
        bad["cell_grid"] = np.asarray(topo["cell_grid"]).copy()
        bad["cell_grid"][3] = int(topo["n_grids"])
    elif mutate == "empty_grid":
        goff = np.asarray(topo["grid_off"]).copy()
        bad["grid_off"] = np.concatenate([goff[:1], goff])   # grid 0 now holds no cells
        bad["n_grids"] = int(topo["n_grids"]) + 1
    elif mutate == "bad_face_dir":
        bad["face_dir"] = np.asarray(topo["face_dir"]).copy()
        bad["face_dir"][0] = 7
    elif mutate == "bad_bc_kind":
        kinds = np.asarray(topo["face_kind"])
        j = int(np.nonzero(kinds == abi.KG_FACE_DOMAIN if hasattr(abi, "KG_FACE_DOMAIN") else kinds == 1)[0][0])
        bad["face_bc_kind"] = np.asarray(topo["face_bc_kind"]).copy()
        bad["face_bc_kind"][j] = 9
    elif mutate == "no_cells":
        bad["n_cells"] = 0
    err = _footprint_error(p, bad)
    assert err.code == code, (mutate, err.code, str(err))
    assert words in str(err), (mutate, str(err))


def test_flattener_rejects_mismatched_params(lib):
    p = cases.collision(center=0.5)
    topo, _ = cases.build(p)
    prm = abi.make_params(p)
    prm.dim = 3
    prm.ndf = 1
    with pytest.raises(S.KitGpuError) as e:
        S.topology_footprint(prm, topo)
    assert e.value.code == 1
