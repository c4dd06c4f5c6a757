"""ABMC / AMC ordering and Reordering on the device (senk_dev_abmc_ordering,
senk_dev_reordering_{d,s}) against the host GetABMCPermutation(..., "simple"),
GetAMCPermutation and Reordering (the product's restatement, pinned to the
reference): identical arrays. At the benchmark's size the whole setup
(ordering, reordering, ILU(0)) runs on the device and is timed beside the
host's."""
import ctypes as C
import time

import numpy as np
import pytest

from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes()


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def dev_ordering(torch, A, bs):
    c, r = _dev(torch, A.cind.astype(np.int32)), _dev(torch, A.rptr.astype(np.int32))
    LP = torch.empty(A.n, dtype=torch.int32, device="cuda")
    RP = torch.empty(A.n, dtype=torch.int32, device="cuda")
    nc = C.c_int(0)
    sc = C.c_void_p()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L.check("ordering", L.lib().senk_dev_abmc_ordering(c.data_ptr(), r.data_ptr(), A.n, bs, C.byref(nc), C.byref(sc),
                                                       LP.data_ptr(), RP.data_ptr(), None))
    ms = (time.perf_counter() - t0) * 1e3
    size_color = np.ctypeslib.as_array(C.cast(sc, C.POINTER(C.c_int)), shape=(nc.value + 1,)).copy()
    L.lib().senk_free(sc)
    return nc.value, size_color, LP, RP, ms


def _shuffled(A, seed):
    p = np.random.default_rng(seed).permutation(A.n).astype(np.int32)
    rp = np.empty_like(p)
    rp[p] = np.arange(A.n, dtype=np.int32)
    return S.Reordering(A, p, rp)


CASES = {
    "poisson128": lambda: P.poisson2d(128),
    "convdiff24": lambda: P.convdiff3d(24, 0.5),
    "vardiff16": lambda: P.vardiff3d(16, 1.5, 4.0, 3),
    "block27_6": lambda: P.block27(6, seed=0),
    "convdiff16_shuffled": lambda: _shuffled(P.convdiff3d(16, 0.5), 1),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("bs", [1, 4, 16])
def test_device_ordering_equals_the_reference(torch, case, bs):
    A = CASES[case]()
    if A.n % bs:
        pytest.skip("N not a multiple of bs")
    nc, sc, LP, RP, _ = dev_ordering(torch, A, bs)
    rnc, rsc, rLP, rRP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bs, False, "simple")
    assert nc == rnc and _same(sc, rsc.astype(np.int32))
    assert _same(LP.cpu().numpy(), rLP.astype(np.int32)) and _same(RP.cpu().numpy(), rRP.astype(np.int32))
    if bs == 1:
        anc, asc, aLP, _ = S.GetAMCPermutation(A.cind, A.rptr, A.n, False)
        assert nc == anc and _same(LP.cpu().numpy(), aLP.astype(np.int32))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("case", ["vardiff16", "block27_6", "convdiff16_shuffled"])
def test_device_reordering_equals_the_reference(torch, case, dtype):
    A = CASES[case]()
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 4 if A.n % 4 == 0 else 1, False, "connect")
    want = S.Reordering(A, LP, RP)
    v, c, r = _dev(torch, A.val.astype(dtype)), _dev(torch, A.cind), _dev(torch, A.rptr)
    ov = torch.empty(A.nnz, dtype=v.dtype, device="cuda")
    oc = torch.empty(A.nnz, dtype=torch.int32, device="cuda")
    orp = torch.empty(A.n + 1, dtype=torch.int32, device="cuda")
    sfx = "s" if dtype == np.float32 else "d"
    LPd, RPd = _dev(torch, LP.astype(np.int32)), _dev(torch, RP.astype(np.int32))  # held until the call has run
    L.check("reordering", getattr(L.lib(), f"senk_dev_reordering_{sfx}")(
        v.data_ptr(), c.data_ptr(), r.data_ptr(), LPd.data_ptr(), RPd.data_ptr(), A.n, ov.data_ptr(), oc.data_ptr(),
        orp.data_ptr(), None))
    assert _same(orp.cpu().numpy(), want.rptr) and _same(oc.cpu().numpy(), want.cind)
    # the values are moved, not computed: FP32 is the FP64 result cast
    assert _same(ov.cpu().numpy(), want.val.astype(dtype))


def test_device_setup_at_benchmark_size(torch):
    """convdiff3d 128^3, simple blocking bsize 16: ordering, reordering and
    ILU(0) on the device equal the host's; times printed."""
    A = P.convdiff3d(128, 0.5)
    t0 = time.perf_counter()
    rnc, rsc, rLP, rRP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "simple")
    Ar = S.Reordering(A, rLP, rRP)
    t_order = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    F = S.Ilu0(Ar)
    t_ilu = (time.perf_counter() - t0) * 1e3
    nc, sc, LP, RP, ms = dev_ordering(torch, A, 16)
    assert nc == rnc and _same(sc, rsc.astype(np.int32)) and _same(LP.cpu().numpy(), rLP.astype(np.int32))
    v, c, r = _dev(torch, A.val), _dev(torch, A.cind), _dev(torch, A.rptr)
    ov = torch.empty(A.nnz, dtype=torch.float64, device="cuda")
    oc = torch.empty(A.nnz, dtype=torch.int32, device="cuda")
    orp = torch.empty(A.n + 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L.check("reordering", L.lib().senk_dev_reordering_d(v.data_ptr(), c.data_ptr(), r.data_ptr(), LP.data_ptr(),
                                                        RP.data_ptr(), A.n, ov.data_ptr(), oc.data_ptr(),
                                                        orp.data_ptr(), None))
    cp = np.ascontiguousarray(sc, np.int32)
    L.check("ilu0", L.lib().senk_dev_ilu0_d(ov.data_ptr(), oc.data_ptr(), orp.data_ptr(), A.n, L.ptr(cp), nc, 16,
                                            None))
    torch.cuda.synchronize()
    t_dev = (time.perf_counter() - t0) * 1e3
    assert _same(orp.cpu().numpy(), Ar.rptr) and _same(oc.cpu().numpy(), Ar.cind)
    assert _same(ov.cpu().numpy(), F.val)
    print(f"128^3 setup, simple ABMC bsize 16 ({nc} colours): host ordering+reordering {t_order:.0f} ms, "
          f"ILU(0) {t_ilu:.0f} ms; device ordering {ms:.1f} ms, reordering+ILU(0) {t_dev:.1f} ms")
