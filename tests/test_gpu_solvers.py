"""GPU solvers through the C ABI against the reference (golden fixtures) and the
oracle: iteration counts within +-2 of the reference with the same ordering and
preconditioner, and the FP64 true residual ||b-Ax||/||b|| below the tolerance."""
import numpy as np
import pytest

from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S
from senk_gb300 import solver as SV

pytestmark = pytest.mark.gpu

ORTHS = [L.ORTH_CGS2, L.ORTH_CGS, L.ORTH_MGS]


@pytest.fixture(scope="module")
def c1():
    A = P.poisson2d(128)
    b = A.matvec(np.ones(A.n))
    return A, b, float(np.linalg.norm(b))


def true_res(port, A, b, x):
    return port.relative_residual(A, b, x)


@pytest.mark.parametrize("orth", ORTHS)
def test_c1_ilu_gmres_natural(port, golden, c1, orth):
    A, b, nb = c1
    L_, U_, _ = S.Split(S.Ilu0(A), "L-DU", True)
    x = np.zeros(A.n)
    r = SV.IluGmresm(A.val, A.cind, A.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, b, x, nb,
                     10000 // 30, 30, A.n, 1e-8, orth=orth)
    assert r.converged and abs(r.iters - golden["c1"]["IluGmresm_m30"]["iters"]) <= 2
    assert r.res <= 1e-8 and true_res(port, A, b, x) < 2e-8


@pytest.mark.parametrize("orth", ORTHS)
def test_c1_abmc_ilu_gmres(port, golden, c1, orth):
    A, b, nb = c1
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    br = b[LP]
    x = np.zeros(A.n)
    r = SV.AbmcIluGmresm(Ar.val, Ar.cind, Ar.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, sc, nc, 16,
                         br, x, nb, 10000 // 30, 30, A.n, 1e-8, orth=orth)
    assert r.converged and abs(r.iters - golden["c1"]["AbmcIluGmresm_m30"]["iters"]) <= 2
    assert true_res(port, Ar, br, x) < 2e-8


def test_c1_amc_ilu_gmres(port, golden, c1):
    A, b, nb = c1
    nc, sc, LP, RP = S.GetAMCPermutation(A.cind, A.rptr, A.n, False)
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    br = b[LP]
    x = np.zeros(A.n)
    r = SV.AmcIluGmresm(Ar.val, Ar.cind, Ar.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, sc, nc, br, x,
                        nb, 10000 // 30, 30, A.n, 1e-8)
    assert r.converged and abs(r.iters - golden["c1"]["AmcIluGmresm_m30"]["iters"]) <= 2
    assert true_res(port, Ar, br, x) < 2e-8


def test_c1_gmres_unpreconditioned(port, golden, c1):
    A, b, nb = c1
    x = np.zeros(A.n)
    r = SV.Gmresm(A.val, A.cind, A.rptr, b, x, nb, 10000 // 30, 30, A.n, 1e-8, orth=L.ORTH_MGS)
    assert r.converged and abs(r.iters - golden["c1"]["Gmresm_m30"]["iters"]) <= 2
    assert true_res(port, A, b, x) < 5e-8


def test_c1_ilu_gmres_float(port, golden, c1):
    A, b, _ = c1
    L_, U_, _ = S.Split(S.Ilu0(A), "L-DU", True)
    x = np.zeros(A.n, np.float32)
    bf = b.astype(np.float32)
    nb = float(np.float32(np.sqrt(np.dot(b, b))))
    r = SV.IluGmresm(A.val, A.cind, A.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, bf, x, nb,
                     10000 // 30, 30, A.n, 1e-6)
    assert r.converged and abs(r.iters - golden["c1"]["IluGmresm_float_m30"]["iters"]) <= 2
    assert true_res(port, A, b, x.astype(np.float64)) < 2e-6


def test_small_golden_solution(port, small, golden):
    s = small
    Ar = P.Csr(s["Ar_val"], s["Ar_cind"], s["Ar_rptr"])
    L_ = P.Csr(s["L_val"], s["L_cind"], s["L_rptr"])
    U_ = P.Csr(s["U_val"], s["U_cind"], s["U_rptr"])
    sc = s["size_color"]
    x = np.zeros(Ar.n)
    r = SV.AbmcIluGmresm(Ar.val, Ar.cind, Ar.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, sc,
                         len(sc) - 1, 16, s["b"], x, float(np.linalg.norm(s["b"])), 100, 30, Ar.n, 1e-8,
                         orth=L.ORTH_MGS)
    assert r.iters == golden["convdiff16"]["AbmcIluGmresm_m30"]["iters"]
    assert np.max(np.abs(x - s["x_gmres"])) <= 1e-10 * np.max(np.abs(s["x_gmres"]))


def test_system_resolve_and_verbose(port, capfd):
    A = P.convdiff3d(24, 0.5)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    b = Ar.matvec(P.uniform_solution(A.n, 0)[LP])
    nb = float(np.linalg.norm(b))
    sysm = SV.System(Ar, L_, U_, L.PC_ILU_ABMC, sc, nc, 16, m_max=30, verbose=True)
    sysm.set_rhs(b)
    r1 = sysm.gmres(nb, 100, 30, 1e-8)
    x1 = sysm.get_x()
    sysm.set_rhs(b)
    r2 = sysm.gmres(nb, 100, 30, 1e-8)
    x2 = sysm.get_x()
    assert r1.iters == r2.iters and np.array_equal(x1, x2)  # deterministic reductions
    out = capfd.readouterr().out
    assert f"I iter {r1.iters}\n# res " in out
    want_x, it, _, _ = port.solve("gmres", Ar, b, L=L_, U=U_, pc=3, cptr=sc, cnum=nc, bsize=16, outer=100, m=30,
                                  eps=1e-8, nrm_b=nb)
    assert abs(r1.iters - it) <= 2
    assert port.relative_residual(Ar, b, x1) < 2e-8
    ms, by = sysm.time_op(L.OP_PRECOND, 3)
    assert ms > 0 and by > 0
    sysm.close()


def test_nonconvergence_reports_outer_times_m(c1):
    A, b, nb = c1
    x = np.zeros(A.n)
    r = SV.Gmresm(A.val, A.cind, A.rptr, b, x, nb, 2, 10, A.n, 1e-8)
    assert not r.converged and r.iters == 20 and r.cycles == 2


@pytest.mark.parametrize("sweep", [L.SWEEP_AUTO, L.SWEEP_COLOURS, L.SWEEP_DATAFLOW, L.SWEEP_COMPACT,
                                   L.SWEEP_WIDE, L.SWEEP_ROWS, L.SWEEP_ROWS_WIDE])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_c1_abmc_sweep_schedules(port, golden, c1, sweep, dtype):
    """Every schedule of the ABMC sweeps (compact chains per colour with one or
    two rows per thread, or with the lanes of a chain holding its rows; row
    slots per colour; one dataflow launch per sweep) in both precisions gives
    the reference's iteration count."""
    A, b, nb = c1
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    br = b[LP]
    sy = SV.System(Ar, L_, U_, L.PC_ILU_ABMC, sc, nc, 16, dtype=dtype, m_max=30, sweep=sweep)
    try:
        sy.set_rhs(br)
        eps = 1e-8 if dtype == np.float64 else 1e-5
        r = sy.gmres(nb, 10000 // 30, 30, eps)
        x = sy.get_x().astype(np.float64)
        assert r.converged
        if dtype == np.float64:
            assert abs(r.iters - golden["c1"]["AbmcIluGmresm_m30"]["iters"]) <= 2
            assert port.relative_residual(Ar, br, x) < 2e-8
        else:
            assert port.relative_residual(Ar, br, x) < 1e-4
    finally:
        sy.close()
