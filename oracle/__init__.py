"""ORACLE — test infrastructure, not product code.

Python access to the two CPU implementations of SenK's Krylov path:

* ``port()``: the plain-C restatement in ``oracle/senk_oracle.c`` (built into
  ``oracle/_build/libsenk_oracle.so``).  It exists on every machine: ``build()``
  compiles it, here and on the GPU host.
* ``ref()``: the reference's own headers compiled by ``oracle/Makefile`` into
  ``oracle/_ref/libsenk_ref.so``; available only where the reference sources were
  present at build time (``None`` otherwise).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker / CPU baseline.
The product library (``senk_gb300``) never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libsenk_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsenk_ref.so")
# The reference's include/ directory, for the live pins; given by the caller
# (build(ref_include=...)) or the SENK_REF_INCLUDE environment variable.
REF_INCLUDE = os.environ.get("SENK_REF_INCLUDE", "")

PC_NONE, PC_ILU, PC_ILU_AMC, PC_ILU_ABMC, PC_ILU_BJ, PC_ILUB, PC_ILUB_ABMC = range(7)
OP_CSR, OP_BCSR = 0, 1

_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_F = C.c_float


def build(ref: bool = True, ref_include: str | None = None) -> None:
    """Compile the C restatement, and the reference shim when the reference's
    include/ directory (ref_include, else SENK_REF_INCLUDE) exists."""
    global REF_INCLUDE
    if ref_include:
        REF_INCLUDE = ref_include
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if ref and REF_INCLUDE and os.path.isdir(REF_INCLUDE):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_INCLUDE={REF_INCLUDE}"], check=True)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _take(lib, p, n, dtype):
    """Copy n items from a malloc'd pointer into numpy, then free it."""
    if not p:
        return None
    ct = {np.float64: C.c_double, np.int32: C.c_int, np.float32: C.c_float}[dtype]
    arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(max(n, 0),)).copy() if n > 0 else np.zeros(0, dtype)
    lib.free_fn(p)
    return arr


class _Result(C.Structure):
    _fields_ = [("iters", C.c_int), ("converged", C.c_int), ("res", C.c_double)]


def _op_struct(T):
    class Op(C.Structure):
        _fields_ = [("kind", C.c_int), ("val", _P), ("cind", _P), ("rptr", _P),
                    ("bnl", C.c_int), ("bnw", C.c_int)]
    class Prec(C.Structure):
        _fields_ = [("kind", C.c_int), ("lval", _P), ("lcind", _P), ("lrptr", _P),
                    ("uval", _P), ("ucind", _P), ("urptr", _P), ("cptr", _P),
                    ("cnum", C.c_int), ("bsize", C.c_int), ("bnum", C.c_int),
                    ("bnl", C.c_int), ("bnw", C.c_int)]
    return Op, Prec


_OpD, _PrecD = _op_struct(np.float64)


def parse_solver_stdout(text: str) -> dict:
    """Parse the reference's convergence lines (senk_gmres.hpp:72-73,
    senk_bicgstab.hpp:63-66, senk_gcr.hpp:48,115): returns iters/res/converged
    and, for GCR, the last restart line."""
    out = {"text": text, "iters": None, "res": None, "converged": False}
    m = re.search(r"^I iter (\d+)$", text, re.M)
    if m:
        out["iters"], out["converged"] = int(m.group(1)), True
        r = re.search(r"^# res ([-+0-9.eE]+)$", text, re.M)
        out["res"] = float(r.group(1)) if r else None
        return out
    m = re.search(r"^# iter (\d+)$", text, re.M)
    if m:  # BiCGStab convergence line, or GMRES non-convergence
        out["iters"] = int(m.group(1))
        r = re.search(r"^# res ([-+0-9.eE]+)$", text, re.M)
        if r:
            out["res"], out["converged"] = float(r.group(1)), True
        return out
    m = re.search(r"^# iter (\d+) \(max\)$", text, re.M)
    if m:
        out["iters"] = int(m.group(1))
        return out
    lines = re.findall(r"^(\d+) ([-+0-9.eE]+)$", text, re.M)
    if lines:  # GCR restart lines: the last one is the stopping test
        out["iters"], out["res"] = int(lines[-1][0]), float(lines[-1][1])
    return out


class _Lib:
    """Shared helpers for both libraries (setup functions keep the same names
    behind a prefix: ``oracle_`` for the port, ``ref_`` for the reference)."""

    prefix = ""

    def __init__(self, path):
        self.lib = C.CDLL(path)
        self.free_fn = getattr(self.lib, self.prefix + "free")
        self.free_fn.argtypes = [_P]

    def set_threads(self, n: int) -> None:
        f = self.fn("set_threads", [_I])
        f(int(n))

    def fn(self, name, argtypes, restype=None):
        f = getattr(self.lib, self.prefix + name)
        f.argtypes = argtypes
        f.restype = restype
        return f

    # ---------------------------------------------------------------- setup
    def abmc_permutation(self, cind, rptr, N, bsize, isSym=False, method="connect"):
        f = self.fn("abmc_permutation", [_P, _P, _P, _P, _P, _P, _I, _I, _I, C.c_char_p],
                    _I if self.prefix == "oracle_" else None)
        nc = C.c_int(0)
        sc, lp, rp = _P(), _P(), _P()
        cind, rptr = _i32(cind), _i32(rptr)
        ret = f(_ptr(cind), _ptr(rptr), C.byref(nc), C.byref(sc), C.byref(lp), C.byref(rp),
                N, bsize, int(isSym), method.encode())
        if ret not in (None, 0):
            raise ValueError("abmc_permutation failed")
        return (nc.value, _take(self, sc.value, nc.value + 1, np.int32),
                _take(self, lp.value, N, np.int32), _take(self, rp.value, N, np.int32))

    def amc_permutation(self, cind, rptr, N, isSym=False):
        f = self.fn("amc_permutation", [_P, _P, _P, _P, _P, _P, _I, _I])
        nc = C.c_int(0)
        sc, lp, rp = _P(), _P(), _P()
        cind, rptr = _i32(cind), _i32(rptr)
        f(_ptr(cind), _ptr(rptr), C.byref(nc), C.byref(sc), C.byref(lp), C.byref(rp), N, int(isSym))
        return (nc.value, _take(self, sc.value, nc.value + 1, np.int32),
                _take(self, lp.value, N, np.int32), _take(self, rp.value, N, np.int32))

    def reordering(self, A, LP, RP):
        f = self.fn("reordering", [_P, _P, _P, _P, _P, _I])
        val, cind, rptr = A.val.copy(), A.cind.copy(), A.rptr.copy()
        LP, RP = _i32(LP), _i32(RP)
        f(_ptr(val), _ptr(cind), _ptr(rptr), _ptr(LP), _ptr(RP), A.n)
        return type(A)(val, cind, rptr)

    def ilu0(self, A):
        f = self.fn("ilu0", [_P, _P, _P, _I], _I if self.prefix == "oracle_" else None)
        val = A.val.astype(np.float64).copy()
        ret = f(_ptr(val), _ptr(A.cind), _ptr(A.rptr), A.n)
        if ret not in (None, 0):
            raise ZeroDivisionError("Ilu0: zero pivot")
        return type(A)(val, A.cind.copy(), A.rptr.copy())

    def _level_fill(self, name, A, p):
        f = self.fn(name, [_P, _P, _P, _I, _I])
        v, c, r = self._to_malloc(A)
        pv, pc, pr = _P(v), _P(c), _P(r)
        f(C.byref(pv), C.byref(pc), C.byref(pr), A.n, p)
        for q in (v, c, r):  # neither implementation frees the input arrays
            self.free_fn(q)
        rptr = _take(self, pr.value, A.n + 1, np.int32)
        nnz = int(rptr[-1])
        return type(A)(_take(self, pv.value, nnz, np.float64), _take(self, pc.value, nnz, np.int32), rptr)

    def ilup(self, A, p):
        return self._level_fill("ilup", A, p)

    def alloc_level_zero(self, A, p):
        return self._level_fill("alloc_level_zero", A, p)

    def _to_malloc(self, A):
        """Copy a CSR into malloc'd buffers (functions that realloc/free them)."""
        libc = C.CDLL(None)
        libc.malloc.restype = _P
        libc.malloc.argtypes = [C.c_size_t]
        out = []
        for a in (A.val.astype(np.float64), _i32(A.cind), _i32(A.rptr)):
            p = libc.malloc(max(a.nbytes, 8))
            C.memmove(p, a.ctypes.data, a.nbytes)
            out.append(p)
        return out

    def alloc_block_zero(self, A, bnl, bnw):
        f = self.fn("alloc_block_zero", [_P, _P, _P, _I, _I, _I], _I if self.prefix == "oracle_" else None)
        v, c, r = self._to_malloc(A)
        pv, pc, pr = _P(v), _P(c), _P(r)
        ret = f(C.byref(pv), C.byref(pc), C.byref(pr), A.n, bnl, bnw)
        if self.prefix == "oracle_":
            if ret < 0:
                raise ValueError("alloc_block_zero: N not a multiple of the block")
            for p in (v, c, r):
                self.free_fn(p)
        rptr = _take(self, pr.value, A.n + 1, np.int32)
        nnz = int(rptr[-1])
        return type(A)(_take(self, pv.value, nnz, np.float64), _take(self, pc.value, nnz, np.int32), rptr)

    def remove_off_diagonal(self, A, bnum):
        """Keep the bnum diagonal blocks of A (RemoveOffDiagonal); returns a new matrix."""
        if self.prefix == "oracle_":
            f = self.fn("remove_off_diagonal", [_P, _P, _P, _I, _I], _I)
            v, c, r = A.val.astype(np.float64).copy(), _i32(A.cind).copy(), _i32(A.rptr).copy()
            nnz = f(_ptr(v), _ptr(c), _ptr(r), A.n, bnum)
            return type(A)(v[:nnz].copy(), c[:nnz].copy(), r)
        f = self.fn("remove_off_diagonal", [_P, _P, _P, _I, _I], None)
        v, c, r = self._to_malloc(A)
        pv, pc, pr = _P(v), _P(c), _P(r)
        f(C.byref(pv), C.byref(pc), C.byref(pr), A.n, bnum)
        rptr = _take(self, pr.value, A.n + 1, np.int32)
        nnz = int(rptr[-1])
        return type(A)(_take(self, pv.value, nnz, np.float64), _take(self, pc.value, nnz, np.int32), rptr)

    def split(self, A, key="L-DU", invDiag=True):
        N = A.n
        pc_ = [_P() for _ in range(7)]
        f = self.fn("split", [_P, _P, _P] + [_P] * 7 + [_I, C.c_char_p, _I],
                    _I if self.prefix == "oracle_" else None)
        val = A.val.astype(np.float64)
        f(_ptr(val), _ptr(A.cind), _ptr(A.rptr), *[C.byref(p) for p in pc_], N, key.encode(), int(invDiag))
        lv, lc, lr, uv, uc, ur, d = [p.value for p in pc_]
        lrp = _take(self, lr, N + 1, np.int32)
        L = type(A)(_take(self, lv, int(lrp[-1]), np.float64), _take(self, lc, int(lrp[-1]), np.int32), lrp)
        U = None
        if ur:
            urp = _take(self, ur, N + 1, np.int32)
            U = type(A)(_take(self, uv, int(urp[-1]), np.float64), _take(self, uc, int(urp[-1]), np.int32), urp)
        D = _take(self, d, N, np.float64) if d else None
        return L, U, D

    def get_diag(self, A):
        if self.prefix == "oracle_":
            f = self.fn("get_diag", [_P, _P, _P, _P, _I])
            d = np.zeros(A.n)
            f(_ptr(np.ascontiguousarray(A.val, np.float64)), _ptr(_i32(A.cind)), _ptr(_i32(A.rptr)), _ptr(d), A.n)
            return d
        f = self.fn("get_diag", [_P, _P, _P, _P, _I])
        dp = _P()
        f(_ptr(np.ascontiguousarray(A.val, np.float64)), _ptr(_i32(A.cind)), _ptr(_i32(A.rptr)), C.byref(dp), A.n)
        return _take(self, dp.value, A.n, np.float64)

    def scaling(self, A, ld, rd):
        f = self.fn("scaling", [_P, _P, _P, _P, _P, _I])
        val = np.array(A.val, np.float64)
        ld, rd = np.ascontiguousarray(ld, np.float64), np.ascontiguousarray(rd, np.float64)
        f(_ptr(val), _ptr(_i32(A.cind)), _ptr(_i32(A.rptr)), _ptr(ld), _ptr(rd), A.n)
        return type(A)(val, A.cind.copy(), A.rptr.copy())

    def expand(self, A, key="L"):
        v, c, r = _P(), _P(), _P()
        args = (_ptr(np.ascontiguousarray(A.val, np.float64)), _ptr(_i32(A.cind)), _ptr(_i32(A.rptr)),
                C.byref(v), C.byref(c), C.byref(r), A.n)
        if self.prefix == "oracle_":
            f = self.fn("expand", [_P, _P, _P, _P, _P, _P, _I, C.c_char], _I)
            if f(*args, key.encode()) != 0:
                raise ValueError("expand: key must be L or U")
        else:
            self.fn("expand", [_P, _P, _P, _P, _P, _P, _I, C.c_char_p])(*args, key.encode())
        rp = _take(self, r.value, A.n + 1, np.int32)
        nnz = int(rp[-1])
        return type(A)(_take(self, v.value, nnz, np.float64), _take(self, c.value, nnz, np.int32), rp)

    def read_matrix_market(self, path, remove_zeros=True):
        """(val, cind, rptr, N, M, symmetric) of the file, or None if rejected."""
        v, c, r = _P(), _P(), _P()
        n, m, sym = C.c_int(0), C.c_int(0), C.c_int(0)
        args = [str(path).encode(), C.byref(v), C.byref(c), C.byref(r), C.byref(n), C.byref(m), C.byref(sym),
                int(remove_zeros)]
        if self.prefix == "oracle_":
            f = self.fn("read_matrix_market", [C.c_char_p, _P, _P, _P, _P, _P, _P, _I], _I)
            ret = f(*args)
        else:
            f = self.fn("read_matrix_market", [C.c_char_p, _P, _P, _P, _P, _P, _P, _I, C.c_char_p, _I], _I)
            self.last_stdout = C.create_string_buffer(1 << 16)
            ret = f(*args, self.last_stdout, 1 << 16)
        if ret != 0:
            return None
        rp = _take(self, r.value, n.value + 1, np.int32)
        nnz = int(rp[-1])
        return (_take(self, v.value, nnz, np.float64), _take(self, c.value, nnz, np.int32), rp, n.value, m.value,
                bool(sym.value))

    def csr2bcsr(self, A, bnl, bnw):
        f = self.fn("csr2bcsr", [_P, _P, _P, _P, _P, _P, _I, _I, _I], _I if self.prefix == "oracle_" else None)
        bv, bc, br = _P(), _P(), _P()
        val = A.val.astype(np.float64)
        ret = f(_ptr(val), _ptr(A.cind), _ptr(A.rptr), C.byref(bv), C.byref(bc), C.byref(br), A.n, bnl, bnw)
        if ret not in (None, 0):
            raise ValueError("csr2bcsr: N not a multiple of the block")
        brp = _take(self, br.value, A.n // bnl + 1, np.int32)
        nb = int(brp[-1])
        return (_take(self, bv.value, nb * bnl * bnw, np.float64), _take(self, bc.value, nb, np.int32), brp)

    def csr2sell(self, A, size):
        f = self.fn("csr2sell", [_P, _P, _P, _P, _P, _P, _I, _I], _I)
        sv, sc, sl = _P(), _P(), _P()
        val = A.val.astype(np.float64)
        nnz = f(_ptr(val), _ptr(A.cind), _ptr(A.rptr), C.byref(sv), C.byref(sc), C.byref(sl), size, A.n)
        ns = (A.n + size - 1) // size
        return (_take(self, sv.value, nnz, np.float64), _take(self, sc.value, nnz, np.int32),
                _take(self, sl.value, ns + 1, np.int32))


class Port(_Lib):
    """The C restatement (oracle/senk_oracle.c)."""

    prefix = "oracle_"

    def __init__(self, path=PORT_SO):
        super().__init__(path)

    @staticmethod
    def _sfx(dtype):
        return "_s" if np.dtype(dtype) == np.float32 else "_d"

    def spmv_csr(self, A, x):
        s = self._sfx(A.val.dtype)
        T = _F if s == "_s" else _D
        f = self.fn("spmv_csr" + s, [_P, _P, _P, _P, _P, _I])
        y = np.empty(A.n, dtype=A.val.dtype)
        x = np.ascontiguousarray(x, dtype=A.val.dtype)
        f(_ptr(A.val), _ptr(A.cind), _ptr(A.rptr), _ptr(x), _ptr(y), A.n)
        return y

    def spmv_bcsr(self, bval, bcind, brptr, x, N, bnl, bnw):
        f = self.fn("spmv_bcsr_d", [_P, _P, _P, _P, _P, _I, _I, _I])
        y = np.empty(N)
        f(_ptr(bval), _ptr(bcind), _ptr(brptr), _ptr(np.ascontiguousarray(x, np.float64)), _ptr(y), N, bnl, bnw)
        return y

    def sptrsv(self, F, x, upper, cptr=None, cnum=0, bsize=0, amc=False, dtype=np.float64):
        """Sequential (cptr None), AMC (amc=True) or ABMC sweep of a split factor."""
        s = self._sfx(dtype)
        side = "u" if upper else "l"
        x = np.ascontiguousarray(x, dtype=dtype)
        y = np.zeros(F.n, dtype=dtype)
        val = F.val.astype(dtype)
        if cptr is None:
            f = self.fn(f"sptrsv_{side}{s}", [_P, _P, _P, _P, _P, _I])
            f(_ptr(val), _ptr(F.cind), _ptr(F.rptr), _ptr(x), _ptr(y), F.n)
        elif amc:
            f = self.fn(f"sptrsv_{side}_amc{s}", [_P, _P, _P, _P, _P, _I, _P, _I])
            f(_ptr(val), _ptr(F.cind), _ptr(F.rptr), _ptr(x), _ptr(y), F.n, _ptr(_i32(cptr)), cnum)
        else:
            f = self.fn(f"sptrsv_{side}_abmc{s}", [_P, _P, _P, _P, _P, _I, _P, _I, _I])
            f(_ptr(val), _ptr(F.cind), _ptr(F.rptr), _ptr(x), _ptr(y), F.n, _ptr(_i32(cptr)), cnum, bsize)
        return y

    def ilu_apply(self, L, U, x, cptr=None, cnum=0, bsize=0, amc=False, dtype=np.float64):
        t = self.sptrsv(L, x, False, cptr, cnum, bsize, amc, dtype)
        return self.sptrsv(U, t, True, cptr, cnum, bsize, amc, dtype)

    def ilub_sweep(self, F, x, upper, bnl, bnw, cptr=None, cnum=0, bsize=0, dtype=np.float64):
        """SptrsvBcsr_l/_u on a BCSR factor F = (bval, bcind, brptr); sequential or
        ABMC (cptr counting blocks of bsize rows); dtype float64 or float32."""
        s = self._sfx(dtype)
        bv, bc, br = (np.ascontiguousarray(F[0], dtype), _i32(F[1]), _i32(F[2]))
        x = np.ascontiguousarray(x, dtype)
        y = np.zeros(x.size, dtype)
        side = "u" if upper else "l"
        if cptr is None:
            f = self.fn(f"sptrsv_bcsr_{side}{s}", [_P, _P, _P, _P, _P, _I, _I, _I])
            f(_ptr(bv), _ptr(bc), _ptr(br), _ptr(x), _ptr(y), x.size, bnl, bnw)
        else:
            f = self.fn(f"sptrsv_bcsr_{side}_abmc{s}", [_P, _P, _P, _P, _P, _I, _P, _I, _I, _I, _I])
            f(_ptr(bv), _ptr(bc), _ptr(br), _ptr(x), _ptr(y), x.size, _ptr(_i32(cptr)), cnum, bsize, bnl, bnw)
        return y

    def ilub_apply(self, Lb, Ub, x, bnl, bnw, cptr=None, cnum=0, bsize=0, dtype=np.float64):
        t = self.ilub_sweep(Lb, x, False, bnl, bnw, cptr, cnum, bsize, dtype)
        return self.ilub_sweep(Ub, t, True, bnl, bnw, cptr, cnum, bsize, dtype)

    def dot(self, x, y):
        f = self.fn("dot_d", [_P, _P, _I], _D)
        x, y = np.ascontiguousarray(x, np.float64), np.ascontiguousarray(y, np.float64)
        return f(_ptr(x), _ptr(y), x.size)

    def nrm2(self, x):
        f = self.fn("nrm2_d", [_P, _I], _D)
        x = np.ascontiguousarray(x, np.float64)
        return f(_ptr(x), x.size)

    def relative_residual(self, A, b, x):
        f = self.fn("relative_residual", [_P, _P, _P, _P, _P, _I], _D)
        return f(_ptr(A.val), _ptr(A.cind), _ptr(A.rptr), _ptr(np.ascontiguousarray(b, np.float64)),
                 _ptr(np.ascontiguousarray(x, np.float64)), A.n)

    def solve(self, method, A, b, x0=None, *, L=None, U=None, pc=PC_NONE, cptr=None, cnum=0,
              bsize=0, bnum=0, bnl=0, bnw=0, op=OP_CSR, outer=100, m=30, max_iter=1000,
              eps=1e-8, nrm_b=None, verbose=False, dtype=np.float64):
        """Run oracle_{gmres,gcr,bicgstab}; returns (x, iters, res, converged)."""
        s = self._sfx(dtype)
        T = _F if s == "_s" else _D
        Op, Prec = _op_struct(dtype)
        keep = []

        def arr(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return _ptr(a)

        opv = Op(op, arr(A.val if op == OP_CSR else A[0], dtype), arr(A.cind if op == OP_CSR else A[1], np.int32),
                 arr(A.rptr if op == OP_CSR else A[2], np.int32), bnl, bnw)
        if L is not None and not hasattr(L, "rptr"):  # BCSR tuple
            lv, lc, lr = L
            uv, uc, ur = U
        else:
            lv, lc, lr = (L.val, L.cind, L.rptr) if L is not None else (None, None, None)
            uv, uc, ur = (U.val, U.cind, U.rptr) if U is not None else (None, None, None)
        prv = Prec(pc, arr(lv, dtype), arr(lc, np.int32), arr(lr, np.int32), arr(uv, dtype),
                   arr(uc, np.int32), arr(ur, np.int32), arr(cptr, np.int32), cnum, bsize, bnum, bnl, bnw)
        N = b.size
        b = np.ascontiguousarray(b, dtype=dtype)
        x = np.zeros(N, dtype) if x0 is None else np.array(x0, dtype=dtype)
        if nrm_b is None:
            nrm_b = float(np.sqrt(np.dot(b.astype(np.float64), b.astype(np.float64))))
        res = _Result()
        if method == "gmres":
            f = self.fn("gmres" + s, [C.POINTER(Op), C.POINTER(Prec), _P, _P, T, _I, _I, _I, T, _I, C.POINTER(_Result)], _I)
            rc = f(C.byref(opv), C.byref(prv), _ptr(b), _ptr(x), nrm_b, outer, m, N, eps, int(verbose), C.byref(res))
        elif method == "gcr":
            f = self.fn("gcr" + s, [C.POINTER(Op), C.POINTER(Prec), _P, _P, T, _I, _I, _I, T, _I, C.POINTER(_Result)], _I)
            rc = f(C.byref(opv), C.byref(prv), _ptr(b), _ptr(x), nrm_b, outer, m, N, eps, int(verbose), C.byref(res))
        elif method == "bicgstab":
            f = self.fn("bicgstab" + s, [C.POINTER(Op), C.POINTER(Prec), _P, _P, T, _I, _I, T, _I, C.POINTER(_Result)], _I)
            rc = f(C.byref(opv), C.byref(prv), _ptr(b), _ptr(x), nrm_b, max_iter, N, eps, int(verbose), C.byref(res))
        else:
            raise ValueError(method)
        if rc != 0:
            raise MemoryError("oracle solver allocation failed")
        return x, res.iters, res.res, bool(res.converged)


class Ref(_Lib):
    """The reference's own headers (oracle/_ref/libsenk_ref.so)."""

    prefix = "ref_"

    def __init__(self, path=REF_SO):
        super().__init__(path)

    def spmv_csr(self, A, x):
        f = self.fn("spmv_csr_d", [_P, _P, _P, _P, _P, _I])
        y = np.empty(A.n)
        f(_ptr(A.val), _ptr(A.cind), _ptr(A.rptr), _ptr(np.ascontiguousarray(x, np.float64)), _ptr(y), A.n)
        return y

    def sptrsv(self, F, x, upper, cptr=None, cnum=0, bsize=0, amc=False):
        side = "u" if upper else "l"
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(F.n)
        if cptr is None:
            f = self.fn(f"sptrsv_{side}_d", [_P, _P, _P, _P, _P, _I])
            f(_ptr(F.val), _ptr(F.cind), _ptr(F.rptr), _ptr(x), _ptr(y), F.n)
        elif amc:
            f = self.fn(f"sptrsv_{side}_amc_d", [_P, _P, _P, _P, _P, _I, _P, _I])
            f(_ptr(F.val), _ptr(F.cind), _ptr(F.rptr), _ptr(x), _ptr(y), F.n, _ptr(_i32(cptr)), cnum)
        else:
            f = self.fn(f"sptrsv_{side}_abmc_d", [_P, _P, _P, _P, _P, _I, _P, _I, _I])
            f(_ptr(F.val), _ptr(F.cind), _ptr(F.rptr), _ptr(x), _ptr(y), F.n, _ptr(_i32(cptr)), cnum, bsize)
        return y

    def ilub_sweep(self, F, x, upper, bnl, bnw, cptr=None, cnum=0, bsize=0):
        bv, bc, br = (np.ascontiguousarray(F[0], np.float64), _i32(F[1]), _i32(F[2]))
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(x.size)
        if cptr is None:
            f = self.fn("sptrsv_bcsr_d", [_I, _P, _P, _P, _P, _P, _I, _I, _I], _I)
            rc = f(int(upper), _ptr(bv), _ptr(bc), _ptr(br), _ptr(x), _ptr(y), x.size, bnl, bnw)
        else:
            f = self.fn("sptrsv_bcsr_abmc_d", [_I, _P, _P, _P, _P, _P, _I, _P, _I, _I, _I, _I], _I)
            rc = f(int(upper), _ptr(bv), _ptr(bc), _ptr(br), _ptr(x), _ptr(y), x.size, _ptr(_i32(cptr)), cnum,
                   bsize, bnl, bnw)
        if rc != 0:
            raise ValueError(f"block shape {bnl}x{bnw} not instantiated in the reference shim")
        return y

    def ilub_apply(self, Lb, Ub, x, bnl, bnw, cptr=None, cnum=0, bsize=0):
        t = self.ilub_sweep(Lb, x, False, bnl, bnw, cptr, cnum, bsize)
        return self.ilub_sweep(Ub, t, True, bnl, bnw, cptr, cnum, bsize)

    def solve_text(self, name, *args):
        """Call a ref_* solver wrapper; returns the reference's captured stdout."""
        buf = C.create_string_buffer(1 << 20)
        f = getattr(self.lib, "ref_" + name)
        conv = []
        for a in args:
            if isinstance(a, np.ndarray):
                conv.append(_ptr(a))
            elif isinstance(a, C._SimpleCData):
                conv.append(a)
            elif isinstance(a, float):
                conv.append(_D(a))
            elif isinstance(a, (bytes, str)):
                conv.append(a.encode() if isinstance(a, str) else a)
            else:
                conv.append(_I(int(a)))
        f.restype = _I
        f(*conv, buf, _I(len(buf)))
        return buf.value.decode()


_port = None
_ref = None


def port(threads: int = 1) -> Port:
    """The C restatement; ``threads=1`` (the default) gives the deterministic
    sequential summation order that parity checks need."""
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        _port = Port()
    _port.set_threads(threads)
    return _port


def ref(threads: int = 1):
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            if not (REF_INCLUDE and os.path.isdir(REF_INCLUDE)):
                return None
            build(ref=True)
        _ref = Ref()
    _ref.set_threads(threads)
    return _ref
