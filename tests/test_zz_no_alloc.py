"""kg_residual_sums_noalloc: the residual sums of residual_check! computed from device
arrays the caller owns, without any device allocation by the library.  It serves callers
that cannot allocate device memory at that point (a runtime whose device memory belongs
to its own pool allocator, or a serving loop that must not let an allocation synchronise
the device).  Checked against the sums kg_step reports for the same step, on two
consecutive calls.  Collected last (zz) so that a failure here comes after every other
GPU test has run."""
import ctypes as C

import numpy as np
import pytest

from kitgpu import abi, cases
from kitgpu.solver import GpuStep, load_library

pytestmark = pytest.mark.gpu


def _noalloc(L):
    f = L.kg_residual_sums_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_residual_matches_step_report():
    import torch
    p = cases.cavity(n=8, nv=16, levels=1)
    topo, state = cases.build(p)
    dim = topo["dim"]
    nw = dim + 2
    fluid = topo["cell_bound_enc"] >= 0
    g = GpuStep(abi.make_params(p, st_check_interval=1), topo)
    g.upload_state(state["f"], state["w"], state["prim"])
    fn = _noalloc(load_library())
    prim_old = state["prim"].reshape(-1, nw)[fluid].copy()
    for call in range(2):
        rep = g.step(p.dt(), call, 1)                 # every step is a check step
        prim_new = g.download_state()["prim"].reshape(-1, nw)[fluid].copy()
        dn = torch.tensor(prim_new, dtype=torch.float64, device="cuda").contiguous()
        do = torch.tensor(prim_old, dtype=torch.float64, device="cuda").contiguous()
        out = torch.full((2 * nw,), np.nan, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = fn(dn.data_ptr(), do.data_ptr(), int(prim_new.shape[0]), dim, out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        ref_res = np.array(rep.sum_res[:nw])
        ref_avg = np.array(rep.sum_avg[:nw])
        assert np.allclose(got[:nw], ref_res, rtol=1e-12, atol=1e-12 * ref_res.max())
        assert np.allclose(got[nw:], ref_avg, rtol=1e-12, atol=1e-12 * ref_avg.max())
        prim_old = prim_new
    g.close()


def _sums_numpy(pn, po):
    d = pn - po
    return np.concatenate([np.sum(d * d, axis=0), np.sum(np.abs(pn), axis=0)])


@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_many_blocks_against_numpy(dim):
    """Sizes that span many scratch rows (3 * 4096 + 17 cells, and about a million), then a
    small call after the large one: the small call reads only the rows it wrote, so the
    large call's leftover rows change nothing.  n_cells = 0 gives zeros."""
    import torch
    fn = _noalloc(load_library())
    nw = dim + 2
    rng = np.random.default_rng(20261203 + dim)
    for n in (3 * 4096 + 17, 1_000_003, 300, 0):
        pn = rng.normal(1.0, 0.5, size=(n, nw))
        po = pn + rng.normal(0.0, 1e-3, size=(n, nw))
        # (an empty input still passes valid pointers: a one-row buffer nothing reads)
        dn = torch.tensor(pn if n else np.ones((1, nw)), dtype=torch.float64, device="cuda").contiguous()
        do = torch.tensor(po if n else np.ones((1, nw)), dtype=torch.float64, device="cuda").contiguous()
        out = torch.full((2 * nw,), np.nan, dtype=torch.float64, device="cuda")
        rc = fn(dn.data_ptr(), do.data_ptr(), n, dim, out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        exp = _sums_numpy(pn, po)
        if n == 0:
            assert np.all(got == 0.0)
        else:
            assert np.allclose(got, exp, rtol=1e-12, atol=0.0), (n, got, exp)


def test_noalloc_rejects_oversized_input():
    fn = _noalloc(load_library())
    # refused before any device work: the size check comes first
    rc = fn(C.c_void_p(16), C.c_void_p(16), 4_194_305, 2, C.c_void_p(16), None)
    assert rc == 1
    buf = C.create_string_buffer(256)
    load_library().kg_last_error(None, buf, 256)
    assert b"exceeds the maximum" in buf.value
