"""ILU(0) factorisation on the GPU (senk_dev_ilu0_d/_s) against the host Ilu0
(include/senk_matrix.hpp:418-448 restated in include/senk_matrix.hpp, itself
pinned to the reference bit for bit): the factors must be identical, bit for
bit, under the natural, AMC and ABMC orders, and at the benchmark's size."""
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


def _dev_ilu0(torch, A, cptr, cnum, bs, dtype=np.float64):
    v = torch.from_numpy(np.ascontiguousarray(A.val.astype(dtype))).cuda()
    c = torch.from_numpy(np.ascontiguousarray(A.cind)).cuda()
    r = torch.from_numpy(np.ascontiguousarray(A.rptr)).cuda()
    cp = None if cptr is None else np.ascontiguousarray(cptr, np.int32)
    fn = L.lib().senk_dev_ilu0_s if dtype == np.float32 else L.lib().senk_dev_ilu0_d
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    code = fn(v.data_ptr(), c.data_ptr(), r.data_ptr(), A.n, L.ptr(cp), cnum, bs, None)
    ms = (time.perf_counter() - t0) * 1e3
    return code, v.cpu().numpy(), ms


def _ilu0_f32(A):
    """Ilu0 (include/senk_matrix.hpp:418-448) in float32 arithmetic, one rounding
    per operation, for small systems."""
    val = A.val.astype(np.float32).copy()
    cind, rptr = A.cind, A.rptr
    for i in range(1, A.n):
        for k in range(rptr[i], rptr[i + 1]):
            c = cind[k]
            if c >= i:
                break
            for l in range(rptr[c], rptr[c + 1]):
                if cind[l] == c:
                    val[k] = np.float32(val[k] / val[l])
                    break
            pos = rptr[c]
            for j in range(k + 1, rptr[i + 1]):
                for l in range(pos, rptr[c + 1]):
                    if cind[l] < cind[j]:
                        continue
                    pos = l
                    if cind[l] == cind[j]:
                        val[j] = np.float32(val[j] - np.float32(val[k] * val[l]))
                        pos += 1
                    break
    return val


def _order(A, sched, bs=16):
    if sched == "natural":
        return A, None, 0, 1
    if sched == "amc":
        nc, sc, LP, RP = S.GetAMCPermutation(A.cind, A.rptr, A.n, False)
        return S.Reordering(A, LP, RP), sc, nc, 1
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bs, False, "connect")
    return S.Reordering(A, LP, RP), sc, nc, bs


@pytest.mark.parametrize("case", ["poisson128", "convdiff24", "vardiff16"])
@pytest.mark.parametrize("sched", ["natural", "amc", "abmc"])
def test_device_ilu0_is_bit_identical(torch, case, sched):
    A = {"poisson128": lambda: P.poisson2d(128), "convdiff24": lambda: P.convdiff3d(24, 0.5),
         "vardiff16": lambda: P.vardiff3d(16, 1.5, 4.0, 3)}[case]()
    Ar, sc, nc, bs = _order(A, sched)
    code, got, _ = _dev_ilu0(torch, Ar, sc, nc, bs)
    assert code == L.OK, L.lib().senk_last_error().decode()
    want = S.Ilu0(Ar).val
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_device_ilu0_fp32_and_benchmark_size(torch):
    """FP32 factors of the 12^3 system equal an FP32 restatement of Ilu0,
    and the 128^3 benchmark system's FP64 factors are bit-identical; the device
    factorisation is timed beside the host one."""
    A = P.convdiff3d(12, 0.5)
    Ar, sc, nc, bs = _order(A, "abmc")
    code, got, _ = _dev_ilu0(torch, Ar, sc, nc, bs, np.float32)
    assert code == L.OK
    assert np.array_equal(got.view(np.uint32), _ilu0_f32(Ar).view(np.uint32))
    A = P.convdiff3d(128, 0.5)
    Ar, sc, nc, bs = _order(A, "abmc")
    code, got, dev_ms = _dev_ilu0(torch, Ar, sc, nc, bs)
    assert code == L.OK
    t0 = time.perf_counter()
    want = S.Ilu0(Ar).val
    host_ms = (time.perf_counter() - t0) * 1e3
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    print(f"ILU(0) 128^3: device {dev_ms:.1f} ms (incl. schedule checks), host {host_ms:.1f} ms")


def test_device_ilu0_rejects_an_order_that_does_not_fit_the_colours(torch):
    A = P.convdiff3d(12, 0.5)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    code, _, _ = _dev_ilu0(torch, A, sc, nc, 16)  # natural order with ABMC colours
    assert code == L.ERR_ARG


def test_device_ilu0_reports_a_zero_pivot(torch):
    A = P.poisson2d(8)
    A.val[A.rptr[0]] = 0.0  # row 0 is not eliminated: its zero diagonal is row 1's pivot
    code, _, _ = _dev_ilu0(torch, A, None, 0, 1)
    assert code == L.ERR_ZERO_PIVOT
