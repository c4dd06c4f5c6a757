"""Solvers through the C ABI, mirroring senk::solver (include/senk_gmres.hpp,
include/senk_gcr.hpp, include/senk_bicgstab.hpp).

The drop-in functions take the reference's arguments in the reference's order
(host numpy arrays; ``x`` is updated in place) and return the ``Result`` that the
reference only prints.  ``System`` is the device-resident form used for repeated
solves (upload once, solve many times).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import (F32, F64, PC_ILU, PC_ILU_ABMC, PC_ILU_AMC, PC_NONE, Options, Result, SystemDesc, check, lib,
                  ptr)
from .problems import Csr


def _opts(orth=0, spmv=0, verbose=False, sweep=0):
    return Options(orth, spmv, int(verbose), sweep)


def _T(x):
    return np.float32 if x.dtype == np.float32 else np.float64


def _arr(a, dtype):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a


def Gmresm(val, cind, rptr, b, x, nrm_b, outer, m, N, epsilon, **opt) -> Result:
    """senk::solver::Gmresm<T> (include/senk_gmres.hpp:33-95); T from x."""
    T = _T(x)
    fn = "senk_gmres_s" if T == np.float32 else "senk_gmres_d"
    r = Result()
    check(fn, getattr(lib(), fn)(ptr(_arr(val, T)), ptr(_arr(cind, np.int32)), ptr(_arr(rptr, np.int32)),
                                 ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N, epsilon, C.byref(_opts(**opt)),
                                 C.byref(r)))
    return r


def IluGmresm(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b, outer, m, N, epsilon,
              **opt) -> Result:
    """senk::solver::IluGmresm<T> (include/senk_gmres.hpp:197-270); T from x."""
    T = _T(x)
    fn = "senk_ilu_gmres_s" if T == np.float32 else "senk_ilu_gmres_d"
    r = Result()
    keep = [_arr(val, T), _arr(cind, np.int32), _arr(rptr, np.int32), _arr(lval, T), _arr(lcind, np.int32),
            _arr(lrptr, np.int32), _arr(uval, T), _arr(ucind, np.int32), _arr(urptr, np.int32), _arr(b, T)]
    check(fn, getattr(lib(), fn)(*[ptr(a) for a in keep], ptr(x), nrm_b, outer, m, N, epsilon,
                                 C.byref(_opts(**opt)), C.byref(r)))
    return r


def AmcIluGmresm(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, cptr, cnum, b, x, nrm_b, outer, m, N,
                 epsilon, **opt) -> Result:
    """senk::solver::AmcIluGmresm<T> (include/senk_gmres.hpp:293-367); T from x."""
    T = _T(x)
    fn = "senk_amc_ilu_gmres_s" if T == np.float32 else "senk_amc_ilu_gmres_d"
    r = Result()
    keep = [_arr(val, T), _arr(cind, np.int32), _arr(rptr, np.int32), _arr(lval, T),
            _arr(lcind, np.int32), _arr(lrptr, np.int32), _arr(uval, T), _arr(ucind, np.int32),
            _arr(urptr, np.int32), _arr(cptr, np.int32)]
    check(fn, getattr(lib(), fn)(*[ptr(a) for a in keep], cnum, ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N,
                                 epsilon, C.byref(_opts(**opt)), C.byref(r)))
    return r


def AbmcIluGmresm(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, cptr, cnum, bsize, b, x, nrm_b, outer,
                  m, N, epsilon, **opt) -> Result:
    """senk::solver::AbmcIluGmresm<T> (include/senk_gmres.hpp:391-465); T from x."""
    T = _T(x)
    fn = "senk_abmc_ilu_gmres_s" if T == np.float32 else "senk_abmc_ilu_gmres_d"
    r = Result()
    keep = [_arr(val, T), _arr(cind, np.int32), _arr(rptr, np.int32), _arr(lval, T), _arr(lcind, np.int32),
            _arr(lrptr, np.int32), _arr(uval, T), _arr(ucind, np.int32), _arr(urptr, np.int32),
            _arr(cptr, np.int32)]
    check(fn, getattr(lib(), fn)(*[ptr(a) for a in keep], cnum, bsize, ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N,
                                 epsilon, C.byref(_opts(**opt)), C.byref(r)))
    return r


def AbmcIluGmresIr(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, cptr, cnum, bsize, b, x, nrm_b,
                   max_outer, m, N, epsilon, inner_tol=1e-4, inner_cycles=2, **opt) -> Result:
    """AbmcIluGmresm's arguments solved by mixed-precision GMRES-IR (FP32 inner
    solves, FP64 refinement stopping on the FP64 true residual)."""
    r = Result()
    keep = [_arr(val, np.float64), _arr(cind, np.int32), _arr(rptr, np.int32), _arr(lval, np.float64),
            _arr(lcind, np.int32), _arr(lrptr, np.int32), _arr(uval, np.float64), _arr(ucind, np.int32),
            _arr(urptr, np.int32), _arr(cptr, np.int32)]
    check("senk_abmc_ilu_gmres_ir_d",
          lib().senk_abmc_ilu_gmres_ir_d(*[ptr(a) for a in keep], cnum, bsize, ptr(_arr(b, np.float64)), ptr(x), nrm_b,
                                         max_outer, m, N, epsilon, inner_tol, inner_cycles, C.byref(_opts(**opt)),
                                         C.byref(r)))
    return r


def _csr_args(T, *arrays):
    """Contiguous copies: value arrays in T, index arrays in int32 (alternating
    val/cind/rptr triples)."""
    out = []
    for k, a in enumerate(arrays):
        out.append(_arr(a, T if k % 3 == 0 else np.int32))
    return out


def _call(fn, *args):
    r = Result()
    check(fn, getattr(lib(), fn)(*args, C.byref(r)))
    return r


def BcsrGmresm(bval, bcind, brptr, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, **opt) -> Result:
    """senk::solver::Gmresm<T,bnl,bnw> (include/senk_gmres.hpp:113-195); T from x."""
    T = _T(x)
    k = _csr_args(T, bval, bcind, brptr)
    return _call("senk_bcsr_gmres" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N,
                 epsilon, bnl, bnw, C.byref(_opts(**opt)))


def BjIluGmresm(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, bnum, b, x, nrm_b, outer, m, N, epsilon,
                **opt) -> Result:
    """senk::solver::BjIluGmresm<T> (include/senk_gmres.hpp:487-580); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr)
    return _call("senk_bj_ilu_gmres" + _sfx(T), *[ptr(a) for a in k], bnum, ptr(_arr(b, T)), ptr(x), nrm_b, outer,
                 m, N, epsilon, C.byref(_opts(**opt)))


def IlubGmresm(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x, nrm_b, outer, m, N, epsilon,
               bnl, bnw, **opt) -> Result:
    """senk::solver::IlubGmresm<T,bnl,bnw> (include/senk_gmres.hpp:582-677); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr)
    return _call("senk_ilub_gmres" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N,
                 epsilon, bnl, bnw, C.byref(_opts(**opt)))


def AbmcIlubGmresm(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, cptr, cnum, bsize, b, x, nrm_b,
                   outer, m, N, epsilon, bnl, bnw, **opt) -> Result:
    """senk::solver::AbmcIlubGmresm<T,bnl,bnw> (include/senk_gmres.hpp:679-776); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr)
    return _call("senk_abmc_ilub_gmres" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(cptr, np.int32)), cnum, bsize,
                 ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N, epsilon, bnl, bnw, C.byref(_opts(**opt)))


def _sfx(T):
    return "_s" if T == np.float32 else "_d"


def Gcrm(val, cind, rptr, b, x, nrm_b, outer, m, N, epsilon, **opt) -> Result:
    """senk::solver::Gcrm<T> (include/senk_gcr.hpp:30-91); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr)
    return _call("senk_gcr" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N, epsilon,
                 C.byref(_opts(**opt)))


def IluGcrm(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b, outer, m, N, epsilon,
            **opt) -> Result:
    """senk::solver::IluGcrm<T> (include/senk_gcr.hpp:93-161); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr)
    return _call("senk_ilu_gcr" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N,
                 epsilon, C.byref(_opts(**opt)))


def IlubGcrm(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x, nrm_b, outer, m, N, epsilon,
             bnl, bnw, **opt) -> Result:
    """senk::solver::IlubGcrm<T,bnl,bnw> (include/senk_gcr.hpp:163-231); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr)
    return _call("senk_ilub_gcr" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(b, T)), ptr(x), nrm_b, outer, m, N,
                 epsilon, bnl, bnw, C.byref(_opts(**opt)))


def Bicgstab(val, cind, rptr, b, x, nrm_b, max_iter, N, epsilon, **opt) -> Result:
    """senk::solver::Bicgstab<T> (include/senk_bicgstab.hpp:29-105); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr)
    return _call("senk_bicgstab" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(b, T)), ptr(x), nrm_b, max_iter, N,
                 epsilon, C.byref(_opts(**opt)))


def IluBicgstab(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b, max_iter, N, epsilon,
                **opt) -> Result:
    """senk::solver::IluBicgstab<T> (include/senk_bicgstab.hpp:107-196); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr)
    return _call("senk_ilu_bicgstab" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(b, T)), ptr(x), nrm_b, max_iter, N,
                 epsilon, C.byref(_opts(**opt)))


def AbmcIluBicgstab(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, cptr, cnum, bsize, b, x, nrm_b,
                    max_iter, N, epsilon, **opt) -> Result:
    """IluBicgstab with the ABMC colour schedule for its sweeps."""
    k = _csr_args(np.float64, val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr)
    return _call("senk_abmc_ilu_bicgstab_d", *[ptr(a) for a in k], ptr(_arr(cptr, np.int32)), cnum, bsize,
                 ptr(_arr(b, np.float64)), ptr(x), nrm_b, max_iter, N, epsilon, C.byref(_opts(**opt)))


def IlubBicgstab(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x, nrm_b, max_iter, N, epsilon,
                 bnl, bnw, **opt) -> Result:
    """senk::solver::IlubBicgstab<T,bnl,bnw> (include/senk_bicgstab.hpp:198-267); T from x."""
    T = _T(x)
    k = _csr_args(T, val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr)
    return _call("senk_ilub_bicgstab" + _sfx(T), *[ptr(a) for a in k], ptr(_arr(b, T)), ptr(x), nrm_b, max_iter,
                 N, epsilon, bnl, bnw, C.byref(_opts(**opt)))


class System:
    """A device-resident system: A (+ split ILU factors and their schedule) uploaded
    once; b and x live on the device between solves."""

    def __init__(self, A: Csr, L=None, U=None, precond: int = PC_NONE, cptr=None, cnum: int = 0,
                 bsize: int = 1, dtype=np.float64, m_max: int = 30, mixed: int = 0, block=(1, 1), **opt):
        """L, U: split ILU factors (Csr), or for PC_ILUB / PC_ILUB_ABMC the BCSR
        factors as (bval, bcind, brptr) tuples with `block` = (bnl, bnw)."""
        self.dtype = np.dtype(dtype)
        T = self.dtype
        self.n = A.n
        self._keep = [_arr(A.val, T), _arr(A.cind, np.int32), _arr(A.rptr, np.int32)]
        d = SystemDesc()
        d.N, d.dtype = A.n, (F32 if T == np.float32 else F64)
        d.val, d.cind, d.rptr = [ptr(a) for a in self._keep]
        d.precond = precond
        if precond != PC_NONE:
            lv, lc, lr = (L.val, L.cind, L.rptr) if isinstance(L, Csr) else L
            uv, uc, ur = (U.val, U.cind, U.rptr) if isinstance(U, Csr) else U
            fac = [_arr(lv, T), _arr(lc, np.int32), _arr(lr, np.int32), _arr(uv, T), _arr(uc, np.int32),
                   _arr(ur, np.int32)]
            d.bnl, d.bnw = block
            self._keep += fac
            d.lval, d.lcind, d.lrptr, d.uval, d.ucind, d.urptr = [ptr(a) for a in fac]
            if cptr is not None:
                cp = _arr(cptr, np.int32)
                self._keep.append(cp)
                d.cptr = ptr(cp)
            d.cnum, d.bsize = cnum, bsize
        d.m_max = m_max
        d.mixed = int(mixed)
        self._h = C.c_void_p()
        check("senk_system_create", lib().senk_system_create(C.byref(self._h), C.byref(d), C.byref(_opts(**opt))))
        self._keep = None

    @property
    def stream(self) -> int:
        return lib().senk_system_stream(self._h)

    @property
    def b_ptr(self) -> int:
        return lib().senk_system_b(self._h)

    @property
    def x_ptr(self) -> int:
        return lib().senk_system_x(self._h)

    def set_rhs(self, b, x0=None):
        b = _arr(b, self.dtype)
        x0 = None if x0 is None else _arr(x0, self.dtype)
        check("senk_system_set_rhs", lib().senk_system_set_rhs(self._h, ptr(b), ptr(x0)))

    def zero_x(self):
        check("senk_system_zero_x", lib().senk_system_zero_x(self._h))

    def get_x(self):
        x = np.empty(self.n, self.dtype)
        check("senk_system_get_x", lib().senk_system_get_x(self._h, ptr(x)))
        return x

    def time_op(self, op: int, reps: int):
        """(ms per run, algorithmic bytes per run) of one op of the solve path,
        timed with CUDA events on the system's stream."""
        ms, by = C.c_double(0), C.c_longlong(0)
        check("senk_system_time_op", lib().senk_system_time_op(self._h, op, reps, C.byref(ms), C.byref(by)))
        return ms.value, by.value

    def gmres(self, nrm_b, outer, m, epsilon) -> Result:
        r = Result()
        check("senk_system_gmres", lib().senk_system_gmres(self._h, nrm_b, outer, m, epsilon, C.byref(r)))
        return r

    def gmres_ir(self, nrm_b, max_outer, m, epsilon, inner_tol=1e-4, inner_cycles=2) -> Result:
        r = Result()
        check("senk_system_gmres_ir", lib().senk_system_gmres_ir(self._h, nrm_b, max_outer, m, epsilon, inner_tol,
                                                                 inner_cycles, C.byref(r)))
        return r

    def _apply(self, name, v):
        v = _arr(v, self.dtype)
        out = np.empty(self.n, self.dtype)
        nb = v.nbytes
        dx, dy = C.c_void_p(), C.c_void_p()
        check("senk_mem_alloc", lib().senk_mem_alloc(C.byref(dx), nb))
        try:
            check("senk_mem_alloc", lib().senk_mem_alloc(C.byref(dy), nb))
            try:
                check("senk_mem_h2d", lib().senk_mem_h2d(dx, ptr(v), nb))
                check(name, getattr(lib(), name)(self._h, dx, dy))
                check("senk_mem_d2h", lib().senk_mem_d2h(ptr(out), dy, nb))
            finally:
                lib().senk_mem_free(dy)
        finally:
            lib().senk_mem_free(dx)
        return out

    def apply_precond(self, v):
        """K v with the system's preconditioner, host vector in and out."""
        return self._apply("senk_system_apply_pc", v)

    def apply_a(self, v):
        """A v with the system's own SpMV format, host vector in and out."""
        return self._apply("senk_system_apply_a", v)

    def gcr_ir(self, nrm_b, max_outer, m, epsilon, inner_tol=1e-4, inner_cycles=2) -> Result:
        """FP64-outer refinement around FP32 GCR(m) (systems created with mixed=1)."""
        r = Result()
        check("senk_system_gcr_ir", lib().senk_system_gcr_ir(self._h, nrm_b, max_outer, m, epsilon, inner_tol,
                                                             inner_cycles, C.byref(r)))
        return r

    def gcr(self, nrm_b, outer, m, epsilon) -> Result:
        r = Result()
        check("senk_system_gcr", lib().senk_system_gcr(self._h, nrm_b, outer, m, epsilon, C.byref(r)))
        return r

    def bicgstab(self, nrm_b, max_iter, epsilon) -> Result:
        r = Result()
        check("senk_system_bicgstab", lib().senk_system_bicgstab(self._h, nrm_b, max_iter, epsilon, C.byref(r)))
        return r

    def close(self):
        if self._h:
            lib().senk_system_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
