"""ctypes binding of libsenk_gpu.so (the C ABI declared in include/senk_gpu.h).

Loading fails loudly when the library is missing: there is no CPU fallback for
any operation of the solver path.  Build it with ``python -m senk_gb300.build``
(or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

OK, ERR_ARG, ERR_CUDA, ERR_ALLOC, ERR_BREAKDOWN, ERR_ZERO_PIVOT = range(6)
ORTH_CGS, ORTH_CGS2, ORTH_MGS = 0, 1, 2
SPMV_AUTO, SPMV_CSR, SPMV_SELL, SPMV_SELL_SIGMA = 0, 1, 2, 3
SWEEP_AUTO, SWEEP_COLOURS, SWEEP_DATAFLOW, SWEEP_COMPACT, SWEEP_PERSISTENT, SWEEP_WIDE = 0, 1, 2, 3, 4, 5
SWEEP_ROWS, SWEEP_ROWS_WIDE = 6, 7
PC_NONE, PC_ILU, PC_ILU_AMC, PC_ILU_ABMC, PC_ILUB, PC_ILUB_ABMC = 0, 1, 2, 3, 4, 5
OP_SPMV, OP_PRECOND, OP_SWEEP_L, OP_SWEEP_U, OP_DOT, OP_MULTIDOT, OP_UPDATE, OP_INNER = 0, 1, 2, 3, 4, 5, 6, 16
F64, F32 = 0, 1

_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_Fl = C.c_float


class SenkError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


class Result(C.Structure):
    _fields_ = [("iters", _I), ("converged", _I), ("res", _D), ("solve_ms", _D), ("breakdown", _I),
                ("cycles", _I), ("h2d_bytes", C.c_longlong), ("d2h_bytes", C.c_longlong),
                ("launches", C.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Options(C.Structure):
    _fields_ = [("orth", _I), ("spmv", _I), ("verbose", _I), ("sweep", _I)]


class SystemDesc(C.Structure):
    _fields_ = [("N", _I), ("dtype", _I), ("val", _P), ("cind", _P), ("rptr", _P), ("precond", _I),
                ("lval", _P), ("lcind", _P), ("lrptr", _P), ("uval", _P), ("ucind", _P), ("urptr", _P),
                ("cptr", _P), ("cnum", _I), ("bsize", _I), ("m_max", _I), ("mixed", _I), ("bnl", _I), ("bnw", _I)]


_lib = None


def lib() -> C.CDLL:
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: build it with `python -m senk_gb300.build`; "
                          "the solver path has no CPU fallback")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    def d(name, args, res=_I):
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res

    d("senk_last_error", [], C.c_char_p)
    d("senk_version", [])
    d("senk_device_count", [])
    d("senk_set_device", [_I])
    d("senk_free", [_P], None)
    Rp, Op = C.POINTER(Result), C.POINTER(Options)
    d("senk_gmres_d", [_P, _P, _P, _P, _P, _D, _I, _I, _I, _D, Op, Rp])
    d("senk_ilu_gmres_d", [_P] * 11 + [_D, _I, _I, _I, _D, Op, Rp])
    d("senk_ilu_gmres_s", [_P] * 11 + [_Fl, _I, _I, _I, _Fl, Op, Rp])
    d("senk_amc_ilu_gmres_d", [_P] * 10 + [_I, _P, _P, _D, _I, _I, _I, _D, Op, Rp])
    d("senk_abmc_ilu_gmres_d", [_P] * 10 + [_I, _I, _P, _P, _D, _I, _I, _I, _D, Op, Rp])
    d("senk_abmc_ilu_gmres_s", [_P] * 10 + [_I, _I, _P, _P, _Fl, _I, _I, _I, _Fl, Op, Rp])
    d("senk_gmres_s", [_P, _P, _P, _P, _P, _Fl, _I, _I, _I, _Fl, Op, Rp])
    d("senk_amc_ilu_gmres_s", [_P] * 10 + [_I, _P, _P, _Fl, _I, _I, _I, _Fl, Op, Rp])
    fd = [_Fl, _I, _I, _I, _Fl]
    d("senk_gcr_s", [_P] * 5 + fd + [Op, Rp])
    d("senk_ilu_gcr_s", [_P] * 11 + fd + [Op, Rp])
    d("senk_bicgstab_s", [_P] * 5 + [_Fl, _I, _I, _Fl, Op, Rp])
    d("senk_ilu_bicgstab_s", [_P] * 11 + [_Fl, _I, _I, _Fl, Op, Rp])
    d("senk_system_create", [C.POINTER(_P), C.POINTER(SystemDesc), Op])
    d("senk_system_destroy", [_P])
    d("senk_system_stream", [_P], _P)
    d("senk_system_b", [_P], _P)
    d("senk_system_x", [_P], _P)
    d("senk_system_set_rhs", [_P, _P, _P])
    d("senk_system_get_x", [_P, _P])
    d("senk_system_zero_x", [_P])
    d("senk_system_gmres", [_P, _D, _I, _I, _D, Rp])
    d("senk_system_time_op", [_P, _I, _I, C.POINTER(_D), C.POINTER(C.c_longlong)])
    d("senk_system_gmres_ir", [_P, _D, _I, _I, _D, _D, _I, Rp])
    d("senk_system_gcr_ir", [_P, _D, _I, _I, _D, _D, _I, Rp])
    d("senk_system_apply_pc", [_P, _P, _P])
    d("senk_system_apply_a", [_P, _P, _P])
    d("senk_dev_ilu0_d", [_P, _P, _P, _I, _P, _I, _I, _P])
    d("senk_dropin_cache", [_I])
    d("senk_dev_ilu0_s", [_P, _P, _P, _I, _P, _I, _I, _P])
    d("senk_abmc_ilu_gmres_ir_d", [_P] * 10 + [_I, _I, _P, _P, _D, _I, _I, _I, _D, _D, _I, Op, Rp])
    gd = [_D, _I, _I, _I, _D]
    d("senk_bcsr_gmres_d", [_P] * 5 + gd + [_I, _I, Op, Rp])
    d("senk_bj_ilu_gmres_d", [_P] * 9 + [_I, _P, _P] + gd + [Op, Rp])
    d("senk_ilub_gmres_d", [_P] * 11 + gd + [_I, _I, Op, Rp])
    d("senk_abmc_ilub_gmres_d", [_P] * 10 + [_I, _I, _P, _P] + gd + [_I, _I, Op, Rp])
    d("senk_gcr_d", [_P] * 5 + gd + [Op, Rp])
    d("senk_ilu_gcr_d", [_P] * 11 + gd + [Op, Rp])
    d("senk_ilub_gcr_d", [_P] * 11 + gd + [_I, _I, Op, Rp])
    bd = [_D, _I, _I, _D]
    d("senk_bicgstab_d", [_P] * 5 + bd + [Op, Rp])
    d("senk_ilu_bicgstab_d", [_P] * 11 + bd + [Op, Rp])
    d("senk_abmc_ilu_bicgstab_d", [_P] * 10 + [_I, _I, _P, _P] + bd + [Op, Rp])
    d("senk_ilub_bicgstab_d", [_P] * 11 + bd + [_I, _I, Op, Rp])
    gs, bs = [_Fl, _I, _I, _I, _Fl], [_Fl, _I, _I, _Fl]
    d("senk_bcsr_gmres_s", [_P] * 5 + gs + [_I, _I, Op, Rp])
    d("senk_bj_ilu_gmres_s", [_P] * 9 + [_I, _P, _P] + gs + [Op, Rp])
    d("senk_ilub_gmres_s", [_P] * 11 + gs + [_I, _I, Op, Rp])
    d("senk_abmc_ilub_gmres_s", [_P] * 10 + [_I, _I, _P, _P] + gs + [_I, _I, Op, Rp])
    d("senk_ilub_gcr_s", [_P] * 11 + gs + [_I, _I, Op, Rp])
    d("senk_ilub_bicgstab_s", [_P] * 11 + bs + [_I, _I, Op, Rp])
    d("senk_system_gcr", [_P, _D, _I, _I, _D, Rp])
    d("senk_system_bicgstab", [_P, _D, _I, _D, Rp])
    d("senk_dev_spmv_csr_d", [_P, _P, _P, _P, _P, _I, _I, _P])
    d("senk_dev_spmv_csr_s", [_P, _P, _P, _P, _P, _I, _I, _P])
    d("senk_dev_spmv_csr_diag_d", [_P, _P, _P, _P, _P, _P, _I, _P])
    d("senk_dev_spmv_bcsr_d", [_P, _P, _P, _P, _P, _I, _I, _I, _P])
    d("senk_dev_spmv_sell_d", [_P, _P, _P, _I, _P, _P, _I, _P])
    d("senk_dev_dot_d", [_P, _P, _I, C.POINTER(_D), _P])
    d("senk_dev_nrm2_d", [_P, _I, C.POINTER(_D), _P])
    d("senk_dev_axpy_d", [_D, _P, _P, _I, _P])
    d("senk_dev_axpby_d", [_D, _P, _D, _P, _I, _P])
    d("senk_dev_axpyz_d", [_D, _P, _P, _P, _I, _P])
    d("senk_dev_scal_d", [_D, _P, _I, _P])
    d("senk_dev_copy_d", [_P, _P, _I, _P])
    d("senk_ilu_plan_create", [C.POINTER(_P), _I, _I, _P, _P, _P, _P, _P, _P, _I, _P, _I, _I])
    d("senk_ilub_plan_create", [C.POINTER(_P), _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _I, _I])
    d("senk_ilu_plan_apply", [_P, _P, _P, _P])
    d("senk_ilu_plan_sweep", [_P, _I, _P, _P, _P])
    d("senk_ilu_plan_destroy", [_P])
    d("senk_ilu_plan_create_sched", [C.POINTER(_P), _I, _I, _P, _P, _P, _P, _P, _P, _I, _P, _I, _I, _I])
    d("senk_ilu_plan_status", [_P, _P])
    d("senk_ilu_plan_test_stall", [_P, _I, _I])
    d("senk_mpnn_num_params", [])
    d("senk_mpnn_create", [C.POINTER(_P), _P, _I])
    d("senk_mpnn_destroy", [_P])
    d("senk_mpnn_get_params", [_P, _P, _I])
    d("senk_mpnn_set_params", [_P, _P, _I])
    d("senk_mpnn_bind", [_P, _P])
    d("senk_mpnn_set_loss", [_P, _I])
    d("senk_mpnn_set_clip", [_P, _Fl])
    d("senk_mpnn_set_step", [_P, _I])
    d("senk_mpnn_loss_grad", [_P, _P, _P, _P, C.POINTER(_D), _P])
    d("senk_mpnn_train_step", [_P, _P, _P, _P, _Fl, C.POINTER(_D)])
    d("senk_mpnn_apply", [_P, _P, _P, _P])
    d("senk_system_set_learned", [_P, _P, _D])
    d("senk_system_learned_fallback", [_P])
    d("senk_dev_gemm_bf16", [_P, _P, _P, _I, _I, _I, _P])
    d("senk_dev_gemm_tn_bf16", [_P, _P, _P, _I, _P])
    d("senk_mem_alloc", [C.POINTER(_P), C.c_size_t])
    d("senk_mem_free", [_P])
    d("senk_mem_h2d", [_P, _P, C.c_size_t])
    d("senk_mem_d2h", [_P, _P, C.c_size_t])
    d("senk_mem_sync", [])
    d("senk_mem_is_device", [_P])
    d("senk_dev_hadprod_d", [_P, _P, _I, _P])
    d("senk_dev_haddiv_d", [_P, _P, _I, _P])
    PP = C.POINTER(_P)
    d("senk_setup_ilu0", [_P, _P, _P, _I])
    d("senk_setup_split", [_P, _P, _P, PP, PP, PP, PP, PP, PP, PP, _I, C.c_char_p, _I])
    d("senk_setup_abmc_permutation", [_P, _P, C.POINTER(_I), PP, PP, PP, _I, _I, _I, C.c_char_p])
    d("senk_setup_amc_permutation", [_P, _P, C.POINTER(_I), PP, PP, PP, _I, _I])
    d("senk_setup_reordering", [_P, _P, _P, _P, _P, _I])
    d("senk_setup_csr2bcsr", [_P, _P, _P, PP, PP, PP, _I, _I, _I])
    d("senk_setup_alloc_block_zero", [PP, PP, PP, _I, _I, _I])
    d("senk_setup_ilup", [PP, PP, PP, _I, _I])
    d("senk_setup_alloc_level_zero", [PP, PP, PP, _I, _I])
    d("senk_setup_remove_off_diagonal", [PP, PP, PP, _I, _I])
    d("senk_io_read_matrix_market", [C.c_char_p, PP, PP, PP, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), _I])
    d("senk_setup_expand", [_P, _P, _P, PP, PP, PP, _I, C.c_char_p])
    d("senk_dev_abmc_ordering", [_P, _P, _I, _I, C.POINTER(_I), PP, _P, _P, _P])
    for sfx in ("d", "s"):
        d(f"senk_dev_reordering_{sfx}", [_P, _P, _P, _P, _P, _I, _P, _P, _P, _P])
        d(f"senk_dev_get_diag_{sfx}", [_P, _P, _P, _P, _I, _P])
        d(f"senk_dev_scaling_{sfx}", [_P, _P, _P, _P, _P, _I, _P])
        d(f"senk_dev_diag_scaling_{sfx}", [_P, _P, _P, _P, _I, _P])


def check(fn: str, code: int) -> int:
    """Raise SenkError for a non-zero status (breakdown is reported, not raised)."""
    if code not in (OK, ERR_BREAKDOWN):
        raise SenkError(fn, code, lib().senk_last_error().decode())
    return code


def ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def exported_symbols(header: str) -> list:
    """Names of the functions declared in a C header of include/ (for tests)."""
    import re
    text = open(header).read()
    return sorted(set(re.findall(r"\b(senk_[a-z0-9_]+)\s*\(", text)))
