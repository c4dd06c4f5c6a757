"""GCR(m), BiCGStab, ILUB (BCSR factor sweeps), block-Jacobi ILU and BCSR GMRES on
the GPU, through the C ABI, against the reference's golden counts and the oracle.

Iteration counts: within +-2 of the reference (GCR: the same restart, as it only
tests the residual at restarts); the FP64 true residual ||b-Ax||/||b|| is
recomputed on the host. ILUB sweeps: within 1e-12 (infinity norm, relative) of
the oracle, which reproduces the reference's BCSR sweeps bit for bit."""
import ctypes as C

import numpy as np
import pytest

from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S
from senk_gb300 import solver as SV

pytestmark = pytest.mark.gpu

M_GCR = 20


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


@pytest.fixture(scope="module")
def c1():
    A = P.poisson2d(128)
    b = A.matvec(np.ones(A.n))
    return A, b, float(np.linalg.norm(b))


@pytest.fixture(scope="module")
def ilub8(c1):
    A = c1[0]
    L_, U_, _ = S.Split(S.Ilu0(S.AllocBlockZero(A, 8, 1)), "L-DU", True)
    return S.Csr2Bcsr(L_, 8, 1), S.Csr2Bcsr(U_, 8, 1)


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def near(it, want, tol=2):
    return abs(it - want) <= tol


# BiCGStab's count moves with the association of its dot products: the
# reference itself, run with 8 OpenMP threads, took between 68 and 75
# iterations on C1 from run to run (70 with one thread). The bar covers that
# spread instead of the ±2 of the other solvers.
BICG_TOL = 5


# ----------------------------------------------------------------- ILUB sweeps

class IlubPlan:
    def __init__(self, bl, bu, N, bnl, bnw, sc=None, nc=0, bs=0):
        self.h = C.c_void_p()
        self.keep = [np.ascontiguousarray(a) for a in (*bl, *bu)]
        cp = None if sc is None else np.ascontiguousarray(sc, np.int32)
        self.keep.append(cp)
        self.code = L.lib().senk_ilub_plan_create(C.byref(self.h), N, bnl, bnw, *[L.ptr(a) for a in self.keep[:6]],
                                                  L.ptr(cp), nc, bs)

    def __del__(self):
        if self.h:
            L.lib().senk_ilu_plan_destroy(self.h)


def _ilub_factors(A, bnl, bnw, bsize=None):
    sc = nc = None
    if bsize:
        nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bsize, False, "connect")
        A = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(S.AllocBlockZero(A, bnl, bnw)), "L-DU", True)
    return S.Csr2Bcsr(L_, bnl, bnw), S.Csr2Bcsr(U_, bnl, bnw), sc, nc


@pytest.mark.parametrize("bnl,bnw", [(1, 1), (2, 1), (2, 2), (3, 3), (4, 1), (4, 2), (4, 4), (8, 1), (8, 2)])
@pytest.mark.parametrize("bsize", [None, 24])
def test_ilub_sweeps(torch, port, bnl, bnw, bsize):
    A = P.convdiff3d(12, 0.5)  # N = 1728
    bl, bu, sc, nc = _ilub_factors(A, bnl, bnw, bsize)
    pl = IlubPlan(bl, bu, A.n, bnl, bnw, sc, nc or 0, bsize or 0)
    if bsize and bnl == 1:
        # Csr2Bcsr gives an empty L row the first entry of the next non-empty
        # row; under ABMC rows 120 and 121 (the first rows of a colour-0 block)
        # are empty, so row 120 takes entry (122, 121) and the reference's
        # sweep reads y[121] before computing it (the output vector's previous
        # contents). The plan refuses such a factor.
        assert pl.code == L.ERR_ARG
        assert "before the schedule has finished it" in L.lib().senk_last_error().decode()
        return
    L.check("plan", pl.code)
    v = np.random.default_rng(9).uniform(-1, 1, A.n)
    xd = torch.from_numpy(v).cuda()
    yd = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    tl = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
    L.check("sweep", L.lib().senk_ilu_plan_sweep(pl.h, 0, xd.data_ptr(), tl.data_ptr(), None))
    torch.cuda.synchronize()
    want_l = port.ilub_sweep(bl, v, False, bnl, bnw, sc, nc or 0, bsize or 0)
    want = port.ilub_sweep(bu, want_l, True, bnl, bnw, sc, nc or 0, bsize or 0)
    assert rel(tl.cpu().numpy(), want_l) <= 1e-12
    assert rel(yd.cpu().numpy(), want) <= 1e-12
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), xd.data_ptr(), None))  # in place
    torch.cuda.synchronize()
    assert rel(xd.cpu().numpy(), want) <= 1e-12


def test_ilub_sweep_golden(torch, small):
    s = small
    bl = (s["Lb_val"], s["Lb_cind"], s["Lb_rptr"])
    bu = (s["Ub_val"], s["Ub_cind"], s["Ub_rptr"])
    sc = s["size_color"]
    N = s["v"].size
    for cp, key in ((None, "y_ilub_seq"), (sc, "y_ilub_abmc")):
        pl = IlubPlan(bl, bu, N, 8, 1, cp, 0 if cp is None else len(sc) - 1, 0 if cp is None else 16)
        L.check("plan", pl.code)
        xd = torch.from_numpy(s["v"]).cuda()
        yd = torch.zeros(N, dtype=torch.float64, device="cuda")
        L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
        torch.cuda.synchronize()
        assert rel(yd.cpu().numpy(), s[key]) <= 1e-12


# -------------------------------------------------------------------- GCR(m)

def test_c1_gcr_unpreconditioned(port, golden, c1):
    A, b, nb = c1
    x = np.zeros(A.n)
    r = SV.Gcrm(A.val, A.cind, A.rptr, b, x, nb, 10000 // M_GCR, M_GCR, A.n, 1e-8)
    assert r.converged and near(r.iters, golden["c1"]["Gcrm_m20"]["iters"], M_GCR)
    assert port.relative_residual(A, b, x) < 1e-8


def test_c1_ilu_gcr(port, golden, c1):
    A, b, nb = c1
    L_, U_, _ = S.Split(S.Ilu0(A), "L-DU", True)
    x = np.zeros(A.n)
    r = SV.IluGcrm(A.val, A.cind, A.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, b, x, nb,
                   10000 // M_GCR, M_GCR, A.n, 1e-8)
    assert r.converged and r.iters == golden["c1"]["IluGcrm_m20"]["iters"]
    assert port.relative_residual(A, b, x) < 1e-8


def test_c1_ilub_gcr(port, golden, c1, ilub8):
    A, b, nb = c1
    bl, bu = ilub8
    x = np.zeros(A.n)
    r = SV.IlubGcrm(A.val, A.cind, A.rptr, *bl, *bu, b, x, nb, 10000 // M_GCR, M_GCR, A.n, 1e-8, 8, 1)
    assert r.converged and r.iters == golden["c1"]["IlubGcrm_8x1_m20"]["iters"]
    assert port.relative_residual(A, b, x) < 1e-8


# ------------------------------------------------------------------ BiCGStab

def test_c1_bicgstab_unpreconditioned(port, golden, c1):
    A, b, nb = c1
    x = np.zeros(A.n)
    r = SV.Bicgstab(A.val, A.cind, A.rptr, b, x, nb, 10000, A.n, 1e-8)
    assert r.converged and near(r.iters, golden["c1"]["Bicgstab"]["iters"], BICG_TOL)
    assert port.relative_residual(A, b, x) < 2e-8


def test_c1_ilu_bicgstab(port, golden, c1):
    A, b, nb = c1
    L_, U_, _ = S.Split(S.Ilu0(A), "L-DU", True)
    x = np.zeros(A.n)
    r = SV.IluBicgstab(A.val, A.cind, A.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, b, x, nb, 10000,
                       A.n, 1e-8)
    assert r.converged and near(r.iters, golden["c1"]["IluBicgstab"]["iters"], BICG_TOL)
    assert r.res < 1e-8 and port.relative_residual(A, b, x) < 2e-8


def test_c1_ilub_bicgstab(port, golden, c1, ilub8):
    A, b, nb = c1
    bl, bu = ilub8
    x = np.zeros(A.n)
    r = SV.IlubBicgstab(A.val, A.cind, A.rptr, *bl, *bu, b, x, nb, 10000, A.n, 1e-8, 8, 1)
    assert r.converged and near(r.iters, golden["c1"]["IlubBicgstab_8x1"]["iters"], BICG_TOL)
    assert port.relative_residual(A, b, x) < 2e-8


def test_convdiff16_abmc_ilu_bicgstab(port, golden, small):
    s = small
    Ar = P.Csr(s["Ar_val"], s["Ar_cind"], s["Ar_rptr"])
    sc = s["size_color"]
    b = s["b"]
    x = np.zeros(Ar.n)
    r = SV.AbmcIluBicgstab(Ar.val, Ar.cind, Ar.rptr, s["L_val"], s["L_cind"], s["L_rptr"], s["U_val"], s["U_cind"],
                           s["U_rptr"], sc, len(sc) - 1, 16, b, x, float(np.linalg.norm(b)), 1000, Ar.n, 1e-8)
    # the ABMC sweep is the sequential sweep on the reordered system
    assert r.converged and near(r.iters, golden["convdiff16"]["IluBicgstab"]["iters"], BICG_TOL)
    assert port.relative_residual(Ar, b, x) < 2e-8


def test_bicgstab_stops_at_max_iter(c1):
    A, b, nb = c1
    x = np.zeros(A.n)
    r = SV.Bicgstab(A.val, A.cind, A.rptr, b, x, nb, 13, A.n, 1e-8)
    assert not r.converged and r.iters == 13


# ------------------------------------------------------- ILUB / BJ / BCSR GMRES

def test_c1_ilub_gmres_8x1(port, golden, c1, ilub8):
    A, b, nb = c1
    bl, bu = ilub8
    x = np.zeros(A.n)
    r = SV.IlubGmresm(A.val, A.cind, A.rptr, *bl, *bu, b, x, nb, 10000 // 30, 30, A.n, 1e-8, 8, 1)
    assert r.converged and near(r.iters, golden["c1"]["IlubGmresm_8x1_m30"]["iters"])
    assert port.relative_residual(A, b, x) < 2e-8


def test_c1_ilub_gmres_2x2(port, golden, c1):
    A, b, nb = c1
    bl, bu, _, _ = _ilub_factors(A, 2, 2)
    x = np.zeros(A.n)
    r = SV.IlubGmresm(A.val, A.cind, A.rptr, *bl, *bu, b, x, nb, 10000 // 30, 30, A.n, 1e-8, 2, 2)
    assert r.converged and near(r.iters, golden["c1"]["IlubGmresm_2x2_m30"]["iters"])
    assert port.relative_residual(A, b, x) < 2e-8


def test_c1_abmc_ilub_gmres(port, golden, c1):
    A, b, nb = c1
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(S.AllocBlockZero(Ar, 8, 1)), "L-DU", True)
    bl, bu = S.Csr2Bcsr(L_, 8, 1), S.Csr2Bcsr(U_, 8, 1)
    br = b[LP]
    x = np.zeros(A.n)
    r = SV.AbmcIlubGmresm(Ar.val, Ar.cind, Ar.rptr, *bl, *bu, sc, nc, 16, br, x, nb, 10000 // 30, 30, A.n, 1e-8, 8,
                          1)
    assert r.converged and near(r.iters, golden["c1"]["AbmcIlubGmresm_8x1_m30"]["iters"])
    assert port.relative_residual(Ar, br, x) < 2e-8


def test_c1_block_jacobi_ilu_gmres(port, golden, c1):
    A, b, nb = c1
    L_, U_, _ = S.Split(S.Ilu0(S.RemoveOffDiagonal(A, 16)), "L-DU", True)
    x = np.zeros(A.n)
    r = SV.BjIluGmresm(A.val, A.cind, A.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, 16, b, x, nb,
                       10000 // 30, 30, A.n, 1e-8)
    assert r.converged and near(r.iters, golden["c1"]["BjIluGmresm_16_m30"]["iters"])
    assert port.relative_residual(A, b, x) < 2e-8


def test_c1_bcsr_gmres(port, golden, c1):
    A, b, nb = c1
    bv, bc, brp = S.Csr2Bcsr(A, 2, 2)
    x = np.zeros(A.n)
    r = SV.BcsrGmresm(bv, bc, brp, b, x, nb, 10000 // 30, 30, A.n, 1e-8, 2, 2, orth=L.ORTH_MGS)
    assert r.converged and near(r.iters, golden["c1"]["BcsrGmresm_2x2_m30"]["iters"])
    assert port.relative_residual(A, b, x) < 5e-8


# ------------------------------------------------------ resident system reuse

def test_system_gcr_and_bicgstab_repeat(port, c1):
    A, b, nb = c1
    L_, U_, _ = S.Split(S.Ilu0(A), "L-DU", True)
    sy = SV.System(A, L_, U_, L.PC_ILU, m_max=0)
    try:
        its = []
        for _ in range(2):
            sy.set_rhs(b)
            r = sy.gcr(nb, 10000 // M_GCR, M_GCR, 1e-8)
            assert r.converged
            its.append(r.iters)
            assert port.relative_residual(A, b, sy.get_x()) < 1e-8
        for _ in range(2):
            sy.set_rhs(b)
            r = sy.bicgstab(nb, 10000, 1e-8)
            assert r.converged
            its.append(r.iters)
            assert port.relative_residual(A, b, sy.get_x()) < 2e-8
        assert its[0] == its[1] and its[2] == its[3]  # deterministic reductions
    finally:
        sy.close()


# ------------------------------------------- FP32 block / block-Jacobi / ILUB

def test_c1_float_block_solvers(port, c1):
    """The T = float forms of Gmresm<T,2,2> (BCSR), BjIluGmresm, IlubGmresm,
    AbmcIlubGmresm, IlubGcrm and IlubBicgstab on the 2D Poisson 128^2 system,
    against the oracle's own FP32 solves of the same method: iteration counts
    within 2 (GMRES), one restart (GCR, which tests at restarts) or 5
    (BiCGStab, whose count moves with the association of its dot products),
    and the true residual."""
    import oracle as O
    A, b, _ = c1
    f32 = np.float32
    bf = b.astype(f32)
    nb = float(np.float32(np.sqrt(np.dot(b, b))))
    eps = 1e-6

    def fresh():
        return np.zeros(A.n, f32)

    def check_res(x, Am=A, bb=bf, bound=5e-6):
        r = bb.astype(np.float64) - port.spmv_csr(Am, x.astype(np.float64))
        assert np.linalg.norm(r) / np.linalg.norm(bb.astype(np.float64)) < bound

    # GMRES(30) on the BCSR matrix (2x2 blocks, MGS as the reference's Gmresm)
    bv, bc, brp = S.Csr2Bcsr(A, 2, 2)
    x = fresh()
    r = SV.BcsrGmresm(bv, bc, brp, bf, x, nb, 10000 // 30, 30, A.n, eps, 2, 2, orth=L.ORTH_MGS)
    _, it, _, _ = port.solve("gmres", (bv, bc, brp), bf, op=O.OP_BCSR, bnl=2, bnw=2, outer=10000 // 30, m=30,
                             eps=eps, nrm_b=nb, dtype=f32)
    assert r.converged and near(r.iters, it), (r.iters, it)
    check_res(x)
    # block-Jacobi ILU(0), 16 blocks
    Lj, Uj, _ = S.Split(S.Ilu0(S.RemoveOffDiagonal(A, 16)), "L-DU", True)
    x = fresh()
    r = SV.BjIluGmresm(A.val, A.cind, A.rptr, Lj.val, Lj.cind, Lj.rptr, Uj.val, Uj.cind, Uj.rptr, 16, bf, x, nb,
                       10000 // 30, 30, A.n, eps)
    _, it, _, _ = port.solve("gmres", A, bf, L=Lj, U=Uj, pc=O.PC_ILU_BJ, bnum=16, outer=10000 // 30, m=30, eps=eps,
                             nrm_b=nb, dtype=f32)
    assert r.converged and near(r.iters, it), (r.iters, it)
    check_res(x)
    # ILUB 8x1: GMRES(30), GCR(20) (FP32 GCR(20) levels off near 1.3e-6 here,
    # in the oracle too, so it runs to 1e-5), BiCGStab
    bl, bu, _, _ = _ilub_factors(A, 8, 1)
    for method, e, call, tol in (
            ("gmres", eps, lambda x, e: SV.IlubGmresm(A.val, A.cind, A.rptr, *bl, *bu, bf, x, nb, 10000 // 30, 30,
                                                      A.n, e, 8, 1), 2),
            ("gcr", 1e-5, lambda x, e: SV.IlubGcrm(A.val, A.cind, A.rptr, *bl, *bu, bf, x, nb, 10000 // M_GCR,
                                                   M_GCR, A.n, e, 8, 1), 2 * M_GCR),
            ("bicgstab", eps, lambda x, e: SV.IlubBicgstab(A.val, A.cind, A.rptr, *bl, *bu, bf, x, nb, 10000, A.n,
                                                           e, 8, 1), 5)):
        x = fresh()
        r = call(x, e)
        kw = dict(outer=10000 // 30, m=30) if method == "gmres" else (
            dict(outer=10000 // M_GCR, m=M_GCR) if method == "gcr" else dict(max_iter=10000))
        _, it, _, conv = port.solve(method, A, bf, L=bl, U=bu, pc=O.PC_ILUB, bnl=8, bnw=1, eps=e, nrm_b=nb,
                                    dtype=f32, **kw)
        assert conv and r.converged and abs(r.iters - it) <= tol, (method, r.iters, it)
        check_res(x, bound=5 * e)
    # ABMC-ordered ILUB 8x1 GMRES(30)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    La, Ua, _ = S.Split(S.Ilu0(S.AllocBlockZero(Ar, 8, 1)), "L-DU", True)
    bla, bua = S.Csr2Bcsr(La, 8, 1), S.Csr2Bcsr(Ua, 8, 1)
    br = bf[LP]
    x = fresh()
    r = SV.AbmcIlubGmresm(Ar.val, Ar.cind, Ar.rptr, *bla, *bua, sc, nc, 16, br, x, nb, 10000 // 30, 30, A.n, eps, 8,
                          1)
    _, it, _, _ = port.solve("gmres", Ar, br, L=bla, U=bua, pc=O.PC_ILUB_ABMC, cptr=sc, cnum=nc, bsize=16, bnl=8,
                             bnw=1, outer=10000 // 30, m=30, eps=eps, nrm_b=nb, dtype=f32)
    assert r.converged and near(r.iters, it), (r.iters, it)
    check_res(x, Ar, br)
