"""The C-ABI library: it loads without a GPU, exports every symbol that
include/senk_gpu.h declares, and reports errors as status codes."""
import ctypes as C
import os

import numpy as np
import pytest

from senk_gb300 import lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "senk_gpu.h")


def test_library_loads_and_exports_every_declared_symbol():
    lib = L.lib()
    names = L.exported_symbols(HEADER)
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_device_count_without_gpu_is_not_an_error():
    assert L.lib().senk_device_count() >= 0
    assert L.lib().senk_version() >= 100


def test_bad_split_key_is_an_argument_error():
    from senk_gb300 import problems as P, setup as S
    A = P.poisson2d(8)
    with pytest.raises(L.SenkError) as e:
        S.Split(A, "X-Y", True)
    assert e.value.code == L.ERR_ARG and "key" in str(e.value)


def test_abmc_size_mismatch_is_an_argument_error():
    from senk_gb300 import problems as P, setup as S
    A = P.poisson2d(10)  # N = 100 is not a multiple of 16
    with pytest.raises(L.SenkError):
        S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")


def test_zero_pivot_is_reported():
    from senk_gb300 import problems as P, setup as S
    A = P.poisson2d(4)
    A = A.copy()
    A.val[A.rptr[0]] = 0.0  # a_00 = 0: row 1 divides by it
    with pytest.raises(L.SenkError) as e:
        S.Ilu0(A)
    assert e.value.code == L.ERR_ZERO_PIVOT


def test_no_cpu_fallback_when_library_missing(monkeypatch, tmp_path):
    monkeypatch.setattr(L, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(L, "_lib", None)
    with pytest.raises(OSError, match="no CPU fallback"):
        L.lib()
