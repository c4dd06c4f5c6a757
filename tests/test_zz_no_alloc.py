"""The allocation-free column dot product (senk_dev_multidot_d_noalloc).

It serves callers that cannot allocate device memory when they call in: an
application whose own pool owns all GPU memory from start-up, or a latency-
critical loop where cudaMalloc could synchronise the device. It must agree with
numpy's dot products and with the allocating entry point senk_dev_dot_d to
rounding, call after call, although every call reuses one fixed scratch array. This file is collected last
so that a run stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from senk_gb300 import lib as L

pytestmark = pytest.mark.gpu


def _noalloc():
    f = L.lib().senk_dev_multidot_d_noalloc
    f.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _dots(torch, Vd, wd, n, nv):
    """Per-column results of the allocating entry point senk_dev_dot_d."""
    out = []
    for k in range(nv):
        d = C.c_double()
        L.check("senk_dev_dot_d", L.lib().senk_dev_dot_d(Vd[k].data_ptr(), wd.data_ptr(), n, C.byref(d), None))
        out.append(d.value)
    return np.array(out)


def test_noalloc_matches_allocating_dot_on_consecutive_calls():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    f = _noalloc()
    rng = np.random.default_rng(2024)
    # two calls in a row with different shapes: the shared scratch must not leak
    # state from one call into the next
    for n, nv in [(1_000_003, 16), (4097, 5)]:
        V = rng.standard_normal((nv, n))
        w = rng.standard_normal(n)
        Vd = torch.from_numpy(V).cuda()
        wd = torch.from_numpy(w).cuda()
        want = _dots(torch, Vd, wd, n, nv)
        out = torch.full((nv,), float("nan"), dtype=torch.float64, device="cuda")
        rc = f(Vd.data_ptr(), n, nv, wd.data_ptr(), n, out.data_ptr(), None)
        assert rc == L.OK, L.lib().senk_last_error().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        scale = np.abs(V * w).sum(axis=1)
        # against an independent host reference and against the allocating entry
        assert np.all(np.abs(got - V @ w) <= 1e-12 * scale)
        assert np.all(np.abs(got - want) <= 1e-12 * scale)


def test_noalloc_rejects_more_columns_than_its_scratch_holds():
    import torch
    f = _noalloc()
    n = 64
    Vd = torch.zeros((17, n), dtype=torch.float64, device="cuda")
    wd = torch.zeros(n, dtype=torch.float64, device="cuda")
    out = torch.zeros(17, dtype=torch.float64, device="cuda")
    rc = f(Vd.data_ptr(), n, 17, wd.data_ptr(), n, out.data_ptr(), None)
    assert rc == L.ERR_ARG
    assert "[1, 16]" in L.lib().senk_last_error().decode()
