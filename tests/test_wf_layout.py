"""The compact chain layout of the dataflow ILU sweep, checked on the CPU.

tests/cpp/wf_emulate.cpp builds the layout with the library's own builder
(senk_gb300/csrc/wf_layout.hpp) and repeats every access of the GPU kernel
k_sweep_wf with its index checked (block slots, gathers, in-chain columns,
dependency lists); its result must equal the oracle's sequential sweep on the
reordered factors (include/senk_sparse.hpp:132-167) to rounding."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from senk_gb300 import problems as P
from senk_gb300 import setup as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("wf") / "libwfemu.so")
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-I", os.path.join(ROOT, "senk_gb300", "csrc"),
           "-I", cuda_inc, os.path.join(ROOT, "tests", "cpp", "wf_emulate.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(out)
    lib.wf_emulate_levels_d.restype = C.c_int
    lib.wf_emulate_levels_d.argtypes = [C.c_int] + [C.c_void_p] * 3 + [C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                                                        C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    for name in ("wf_cp_schedule_s", "wf_cp_schedule_d"):
        f = getattr(lib, name)
        f.restype = C.c_int
        f.argtypes = [C.c_int] + [C.c_void_p] * 3 + [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_char_p,
                                                      C.c_int]
    for name in ("wf_emulate_d", "wf_emulate_s", "wf_emulate_rl_d", "wf_emulate_rl_s"):
        f = getattr(lib, name)
        f.restype = C.c_int
        f.argtypes = [C.c_int] + [C.c_void_p] * 3 + [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                      C.c_char_p, C.c_int]
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _run(emu, F, upper, sc, nc, bs, x, rl=False):
    T = F.val.dtype
    y = np.zeros_like(x)
    err = C.create_string_buffer(256)
    if rl:
        f = emu.wf_emulate_rl_s if T == np.float32 else emu.wf_emulate_rl_d
    else:
        f = emu.wf_emulate_s if T == np.float32 else emu.wf_emulate_d
    keep = [np.ascontiguousarray(a) for a in (F.val, F.cind, F.rptr, np.asarray(sc, np.int32), x)]
    rc = f(F.n, _p(keep[0]), _p(keep[1]), _p(keep[2]), int(upper), _p(keep[3]), nc, bs, _p(keep[4]), _p(y), err, 256)
    assert rc == 0, err.value.decode()
    return y


CASES = [("convdiff", 16, 16), ("convdiff", 16, 2), ("convdiff", 12, 32), ("poisson", 64, 8), ("vardiff", 16, 4),
         ("convdiff", 12, 1)]


@pytest.mark.parametrize("kind,n,bs", CASES)
def test_emulated_dataflow_sweep_matches_the_oracle(emu, port, kind, n, bs):
    A = {"convdiff": lambda: P.convdiff3d(n, 0.5), "poisson": lambda: P.poisson2d(n),
         "vardiff": lambda: P.vardiff3d(n, 1.5, 4.0, 3)}[kind]()
    if bs == 1:
        nc, sc, LP, RP = S.GetAMCPermutation(A.cind, A.rptr, A.n, False)
    else:
        nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bs, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    v = np.random.default_rng(7).uniform(-1, 1, A.n)
    tl = _run(emu, L_, False, sc, nc, bs, v)
    want_l = port.sptrsv(L_, v, False)
    assert np.max(np.abs(tl - want_l)) <= 1e-14 * np.max(np.abs(want_l))
    t = _run(emu, U_, True, sc, nc, bs, want_l)
    want = port.sptrsv(U_, want_l, True)
    assert np.max(np.abs(t - want)) <= 1e-14 * np.max(np.abs(want))
    # FP32 factors
    L32, U32 = L_.astype(np.float32), U_.astype(np.float32)
    v32 = v.astype(np.float32)
    t32 = _run(emu, U32, True, sc, nc, bs, _run(emu, L32, False, sc, nc, bs, v32))
    want32 = port.ilu_apply(L32, U32, v32, dtype=np.float32)
    assert np.max(np.abs(t32 - want32)) <= 1e-5 * np.max(np.abs(want32))


@pytest.mark.parametrize("kind,n,bs", CASES)
def test_emulated_row_per_lane_sweep_matches_the_oracle(emu, port, kind, n, bs):
    """The chain-major layout and the row-per-lane kernel's accesses
    (k_sweep_rl: chain streams at q*emax, in-chain offsets from the chain
    descriptor, lane-scan offsets, bs - 1 lockstep recurrence steps with U's
    scaled broadcast), repeated on the CPU with every index checked and rows of
    a colour readable only after the colour; the result equals the oracle's
    sequential sweep bit for bit, FP64 and FP32: each row subtracts the same
    products in the same order (entries of earlier colours, then in-chain ones
    in column order) and U scales by the same inverted diagonal."""
    A = {"convdiff": lambda: P.convdiff3d(n, 0.5), "poisson": lambda: P.poisson2d(n),
         "vardiff": lambda: P.vardiff3d(n, 1.5, 4.0, 3)}[kind]()
    if bs == 1:
        nc, sc, LP, RP = S.GetAMCPermutation(A.cind, A.rptr, A.n, False)
    else:
        nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bs, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    v = np.random.default_rng(11).uniform(-1, 1, A.n)
    tl = _run(emu, L_, False, sc, nc, bs, v, rl=True)
    want_l = port.sptrsv(L_, v, False)
    assert np.array_equal(tl, want_l)
    t = _run(emu, U_, True, sc, nc, bs, want_l, rl=True)
    want = port.sptrsv(U_, want_l, True)
    assert np.array_equal(t, want)
    L32, U32 = L_.astype(np.float32), U_.astype(np.float32)
    v32 = v.astype(np.float32)
    t32 = _run(emu, U32, True, sc, nc, bs, _run(emu, L32, False, sc, nc, bs, v32, rl=True), rl=True)
    want32 = port.ilu_apply(L32, U32, v32, dtype=np.float32)
    assert np.array_equal(t32, want32)


def _levels(F, upper):
    """Level sets of a triangular factor (the natural order's schedule): rows in
    processing order and the position range of each level."""
    n = F.n
    lev = np.zeros(n, np.int64)
    rng = range(n - 1, -1, -1) if upper else range(n)
    for i in rng:
        js = F.cind[F.rptr[i] + (1 if upper else 0):F.rptr[i + 1]]
        if js.size:
            lev[i] = lev[js].max() + 1
    order = np.argsort(lev, kind="stable").astype(np.int32)
    ptr = np.concatenate([[0], np.cumsum(np.bincount(lev))]).astype(np.int32)
    return order, ptr


@pytest.mark.parametrize("n", [16, 40])
def test_emulated_level_set_layout_matches_the_oracle(emu, port, n):
    """The natural order's level sets as chains of one row (row map), as the
    single-CTA sweep of small systems uses them."""
    A = P.poisson2d(n)
    L_, U_, _ = S.Split(S.Ilu0(A), "L-DU", True)
    v = np.random.default_rng(3).uniform(-1, 1, A.n)
    out = v
    for F, upper in ((L_, False), (U_, True)):
        order, ptr = _levels(F, upper)
        y = np.zeros(A.n)
        err = C.create_string_buffer(256)
        keep = [np.ascontiguousarray(a) for a in (F.val, F.cind, F.rptr, ptr, order, out)]
        rc = emu.wf_emulate_levels_d(A.n, _p(keep[0]), _p(keep[1]), _p(keep[2]), int(upper), _p(keep[3]),
                                     len(ptr) - 1, _p(keep[4]), _p(keep[5]), _p(y), err, 256)
        assert rc == 0, err.value.decode()
        out = y
    want = port.sptrsv(U_, port.sptrsv(L_, v, False), True)
    assert np.max(np.abs(out - want)) <= 1e-14 * np.max(np.abs(want))


@pytest.mark.parametrize("n,bs,grid", [(24, 16, 7), (24, 16, 1), (32, 4, 150), (16, 1, 13), (64, 16, 456)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_cooperative_schedule(emu, n, bs, grid, dtype):
    """k_sweep_cp's walk on `grid` CTAs (capped at the widest colour, as the
    host does): staging buffers, copy alignment, each group solved once after
    the colours before it."""
    A = P.convdiff3d(n, 0.5)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bs, False, "connect")
    L_, U_, _ = S.Split(S.Ilu0(S.Reordering(A, LP, RP)), "L-DU", True)
    widest = int(np.max(np.diff(np.asarray(sc)) + 31) // 32)
    f = emu.wf_cp_schedule_s if dtype == np.float32 else emu.wf_cp_schedule_d
    for F, upper in ((L_, 0), (U_, 1)):
        keep = [np.ascontiguousarray(a) for a in (F.val.astype(dtype), F.cind, F.rptr, np.asarray(sc, np.int32))]
        err = C.create_string_buffer(256)
        rc = f(F.n, _p(keep[0]), _p(keep[1]), _p(keep[2]), upper, _p(keep[3]), nc, bs, min(grid, widest), err, 256)
        assert rc == 0, err.value.decode()
