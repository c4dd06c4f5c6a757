"""Host-side checks of the ILUB plan (no GPU work: the factors are rejected
before anything is uploaded)."""
import ctypes as C

import numpy as np

from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S


def _create(bl, bu, N, bnl, bnw, sc=None, nc=0, bs=0):
    h = C.c_void_p()
    keep = [np.ascontiguousarray(a) for a in (*bl, *bu)]
    cp = None if sc is None else np.ascontiguousarray(sc, np.int32)
    code = L.lib().senk_ilub_plan_create(C.byref(h), N, bnl, bnw, *[L.ptr(a) for a in keep], L.ptr(cp), nc, bs)
    return code, L.lib().senk_last_error().decode()


def _factors(A, bnl, bnw):
    L_, U_, _ = S.Split(S.Ilu0(S.AllocBlockZero(A, bnl, bnw)), "L-DU", True)
    return S.Csr2Bcsr(L_, bnl, bnw), S.Csr2Bcsr(U_, bnl, bnw)


def test_ilub_plan_rejects_unsupported_shapes_and_sizes():
    A = P.convdiff3d(6, 0.5)  # N = 216
    bl, bu = _factors(A, 8, 1)
    code, msg = _create(bl, bu, A.n, 3, 2)
    assert code == L.ERR_ARG and "not built" in msg
    code, msg = _create(bl, bu, A.n - 1, 8, 1)
    assert code == L.ERR_ARG and "multiple of bnl" in msg


def test_ilub_plan_rejects_a_schedule_the_factors_do_not_fit():
    A = P.convdiff3d(8, 0.5)  # N = 512
    bl, bu = _factors(A, 8, 1)
    # natural-order factors under an ABMC colouring of the same matrix: a block
    # row of an early colour reads rows of a later one
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    code, msg = _create(bl, bu, A.n, 8, 1, sc, nc, 16)
    assert code == L.ERR_ARG and "before the schedule has finished it" in msg
    # bsize that is not a multiple of bnl
    code, msg = _create(bl, bu, A.n, 8, 1, sc, nc, 12)
    assert code == L.ERR_ARG and "multiple of bnl" in msg


def test_ilub_plan_rejects_a_u_factor_without_its_diagonal_square():
    A = P.convdiff3d(8, 0.5)
    bl, bu = _factors(A, 8, 1)
    bv, bc, br = (a.copy() for a in bu)
    bc[br[0]] = bc[br[0] + 1]  # first block of block row 0 no longer the diagonal column 0
    code, msg = _create(bl, (bv, bc, br), A.n, 8, 1)
    assert code == L.ERR_ARG and "diagonal square" in msg


def test_remove_off_diagonal_matches_the_oracle(port):
    A = P.poisson2d(32)
    a, b = S.RemoveOffDiagonal(A, 8), port.remove_off_diagonal(A, 8)
    assert np.array_equal(a.rptr, b.rptr) and np.array_equal(a.cind, b.cind) and np.array_equal(a.val, b.val)
    # twice in a row: the buffers handed back must be owned exactly once
    a2 = S.RemoveOffDiagonal(a, 16)
    assert a2.nnz < a.nnz
