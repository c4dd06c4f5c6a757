"""Host setup of the solver path through the C ABI (numpy in, numpy out).

Mirrors senk::matrix and senk::graph (include/senk_matrix.hpp,
include/senk_graph.hpp): the same functions, argument meanings and outputs as
the reference, returned as arrays instead of malloc'd out-parameters.  Errors
that make the reference exit(1) raise ``SenkError`` here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import SenkError, check, lib, ptr
from .problems import Csr

_P = C.c_void_p


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _take(p, n, dtype):
    """Copy n items from a library-malloc'd pointer, then release it."""
    if not p:
        return None
    ct = {np.dtype(np.float64): C.c_double, np.dtype(np.int32): C.c_int}[np.dtype(dtype)]
    out = np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n,)).copy() if n > 0 else np.zeros(0, dtype)
    lib().senk_free(p)
    return out


def _malloc_copy(a):
    """A malloc'd copy (for functions that free or realloc their input)."""
    libc = C.CDLL(None)
    libc.malloc.restype = _P
    libc.malloc.argtypes = [C.c_size_t]
    p = libc.malloc(max(a.nbytes, 8))
    C.memmove(p, a.ctypes.data, a.nbytes)
    return p


def Ilu0(A: Csr) -> Csr:
    """ILU(0) factors in A's pattern (senk::matrix::Ilu0); returns a new matrix."""
    val = _f64(A.val).copy()
    cind, rptr = _i32(A.cind), _i32(A.rptr)
    check("senk_setup_ilu0", lib().senk_setup_ilu0(ptr(val), ptr(cind), ptr(rptr), A.n))
    return Csr(val, cind.copy(), rptr.copy())


def Split(A: Csr, key: str = "L-DU", invDiag: bool = True):
    """(L, U, diag) as senk::matrix::Split returns them (U/diag may be None)."""
    N = A.n
    outs = [_P() for _ in range(7)]
    val, cind, rptr = _f64(A.val), _i32(A.cind), _i32(A.rptr)
    check("senk_setup_split", lib().senk_setup_split(ptr(val), ptr(cind), ptr(rptr), *[C.byref(o) for o in outs],
                                                     N, key.encode(), int(invDiag)))
    lv, lc, lr, uv, uc, ur, d = [o.value for o in outs]
    lrp = _take(lr, N + 1, np.int32)
    L = Csr(_take(lv, int(lrp[-1]), np.float64), _take(lc, int(lrp[-1]), np.int32), lrp)
    U = None
    if ur:
        urp = _take(ur, N + 1, np.int32)
        U = Csr(_take(uv, int(urp[-1]), np.float64), _take(uc, int(urp[-1]), np.int32), urp)
    D = _take(d, N, np.float64) if d else None
    return L, U, D


def GetABMCPermutation(cind, rptr, N: int, bsize: int, isSym: bool = False, bmethod: str = "connect"):
    """(num_color, size_color, LP, RP) of senk::graph::GetABMCPermutation."""
    nc = C.c_int(0)
    sc, lp, rp = _P(), _P(), _P()
    cind, rptr = _i32(cind), _i32(rptr)
    check("senk_setup_abmc_permutation",
          lib().senk_setup_abmc_permutation(ptr(cind), ptr(rptr), C.byref(nc), C.byref(sc), C.byref(lp),
                                            C.byref(rp), N, bsize, int(isSym), bmethod.encode()))
    return nc.value, _take(sc.value, nc.value + 1, np.int32), _take(lp.value, N, np.int32), _take(rp.value, N, np.int32)


def GetAMCPermutation(cind, rptr, N: int, isSym: bool = False):
    """(num_color, size_color, LP, RP) of senk::graph::GetAMCPermutation."""
    nc = C.c_int(0)
    sc, lp, rp = _P(), _P(), _P()
    cind, rptr = _i32(cind), _i32(rptr)
    check("senk_setup_amc_permutation",
          lib().senk_setup_amc_permutation(ptr(cind), ptr(rptr), C.byref(nc), C.byref(sc), C.byref(lp),
                                           C.byref(rp), N, int(isSym)))
    return nc.value, _take(sc.value, nc.value + 1, np.int32), _take(lp.value, N, np.int32), _take(rp.value, N, np.int32)


def Reordering(A: Csr, LP, RP) -> Csr:
    """P A P^T (senk::matrix::Reordering with LP and RP); returns a new matrix."""
    val, cind, rptr = _f64(A.val).copy(), _i32(A.cind).copy(), _i32(A.rptr).copy()
    check("senk_setup_reordering", lib().senk_setup_reordering(ptr(val), ptr(cind), ptr(rptr), ptr(_i32(LP)),
                                                               ptr(_i32(RP)), A.n))
    return Csr(val, cind, rptr)


def Csr2Bcsr(A: Csr, bnl: int, bnw: int):
    """(bval, bcind, brptr) of senk::matrix::Csr2Bcsr."""
    bv, bc, br = _P(), _P(), _P()
    val, cind, rptr = _f64(A.val), _i32(A.cind), _i32(A.rptr)
    check("senk_setup_csr2bcsr", lib().senk_setup_csr2bcsr(ptr(val), ptr(cind), ptr(rptr), C.byref(bv),
                                                           C.byref(bc), C.byref(br), A.n, bnl, bnw))
    brp = _take(br.value, A.n // bnl + 1, np.int32)
    nb = int(brp[-1])
    return _take(bv.value, nb * bnl * bnw, np.float64), _take(bc.value, nb, np.int32), brp


def _realloc_call(fn, A: Csr, *args) -> Csr:
    pv, pc, pr = _P(_malloc_copy(_f64(A.val))), _P(_malloc_copy(_i32(A.cind))), _P(_malloc_copy(_i32(A.rptr)))
    olds = (pv.value, pc.value, pr.value)
    check(fn, getattr(lib(), fn)(C.byref(pv), C.byref(pc), C.byref(pr), A.n, *args))
    rptr = _take(pr.value, A.n + 1, np.int32)
    nnz = int(rptr[-1])
    out = Csr(_take(pv.value, nnz, np.float64), _take(pc.value, nnz, np.int32), rptr)
    return out, olds


def AllocBlockZero(A: Csr, bnl: int, bnw: int) -> Csr:
    """senk::matrix::AllocBlockZero (frees its input, like the reference)."""
    out, _ = _realloc_call("senk_setup_alloc_block_zero", A, bnl, bnw)
    return out


def Ilup(A: Csr, p: int) -> Csr:
    """senk::matrix::Ilup (the reference leaves its input allocated; freed here)."""
    out, olds = _realloc_call("senk_setup_ilup", A, p)
    for q in olds:
        lib().senk_free(q)
    return out


def AllocLevelZero(A: Csr, p: int) -> Csr:
    """senk::matrix::AllocLevelZero (input freed here, see Ilup)."""
    out, olds = _realloc_call("senk_setup_alloc_level_zero", A, p)
    for q in olds:
        lib().senk_free(q)
    return out


def RemoveOffDiagonal(A: Csr, bnum: int) -> Csr:
    """senk::matrix::RemoveOffDiagonal: keep the bnum diagonal blocks of N/bnum
    rows. It reallocates val and cind and edits rptr in place, so the input
    buffers are the output's (nothing else to free)."""
    out, _ = _realloc_call("senk_setup_remove_off_diagonal", A, bnum)
    return out


def ReadMatrixMarket(path, removeZeros: bool = True):
    """senk::io::ReadMatrixMarket: (Csr of the stored entries, M, symmetric).
    A symmetric file gives its stored triangle; Expand(A, "L") makes the full
    matrix, as the reference's driver does."""
    pv, pc, pr = _P(), _P(), _P()
    n, m, sym = C.c_int(0), C.c_int(0), C.c_int(0)
    check("senk_io_read_matrix_market",
          lib().senk_io_read_matrix_market(str(path).encode(), C.byref(pv), C.byref(pc), C.byref(pr), C.byref(n),
                                           C.byref(m), C.byref(sym), int(removeZeros)))
    rptr = _take(pr.value, n.value + 1, np.int32)
    nnz = int(rptr[-1])
    return Csr(_take(pv.value, nnz, np.float64), _take(pc.value, nnz, np.int32), rptr), m.value, bool(sym.value)


def Expand(A: Csr, key: str = "L") -> Csr:
    """senk::matrix::Expand: the full matrix from its stored triangle."""
    pv, pc, pr = _P(), _P(), _P()
    check("senk_setup_expand", lib().senk_setup_expand(ptr(_f64(A.val)), ptr(_i32(A.cind)), ptr(_i32(A.rptr)),
                                                       C.byref(pv), C.byref(pc), C.byref(pr), A.n, key.encode()))
    rptr = _take(pr.value, A.n + 1, np.int32)
    nnz = int(rptr[-1])
    return Csr(_take(pv.value, nnz, np.float64), _take(pc.value, nnz, np.int32), rptr)


__all__ = ["Ilu0", "Split", "GetABMCPermutation", "GetAMCPermutation", "Reordering", "Csr2Bcsr",
           "AllocBlockZero", "Ilup", "AllocLevelZero", "RemoveOffDiagonal", "ReadMatrixMarket", "Expand",
           "SenkError"]
