"""Mixed-precision GMRES-IR (FP32 inner solves, FP64 refinement): the FP64 true
residual ||b - Ax|| / ||b|| must fall below the tolerance, and the inner solves
must need about as many iterations as the plain FP64 solve."""
import numpy as np
import pytest

from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S
from senk_gb300 import solver as SV

pytestmark = pytest.mark.gpu


def abmc_system(A, xt, bsize=16):
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bsize, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    return Ar, L_, U_, sc, nc, Ar.matvec(xt[LP])


@pytest.mark.parametrize("case,eps", [("poisson128", 1e-8), ("poisson128", 1e-10), ("convdiff32", 1e-8),
                                      ("vardiff32", 1e-10)])
def test_gmres_ir_reaches_fp64_true_residual(port, case, eps):
    A = {"poisson128": lambda: P.poisson2d(128), "convdiff32": lambda: P.convdiff3d(32, 0.5),
         "vardiff32": lambda: P.vardiff3d(32, 1.5, 8.0, 0)}[case]()
    xt = P.normal_solution(A.n, 1) if case == "vardiff32" else P.uniform_solution(A.n, 0)
    Ar, L_, U_, sc, nc, b = abmc_system(A, xt)
    nb = float(np.linalg.norm(b))
    m = 50 if case == "vardiff32" else 30
    sysm = SV.System(Ar, L_, U_, L.PC_ILU_ABMC, sc, nc, 16, m_max=m, mixed=True)
    sysm.set_rhs(b)
    r = sysm.gmres_ir(nb, 20, m, eps, 1e-4, 4)
    x = sysm.get_x()
    tr = port.relative_residual(Ar, b, x)
    assert r.converged and r.res <= eps and tr <= eps * 1.01
    assert 1 <= r.cycles <= 8
    # the plain FP64 solve of the same system, for comparison
    sysm.zero_x()
    rp = sysm.gmres(nb, 10000 // m, m, eps)
    assert rp.converged
    assert r.iters <= 2.5 * rp.iters + 2 * m
    sysm.close()


def test_gmres_ir_dropin_entry(port):
    A = P.convdiff3d(24, 0.5)
    xt = P.uniform_solution(A.n, 0)
    Ar, L_, U_, sc, nc, b = abmc_system(A, xt)
    nb = float(np.linalg.norm(b))
    x = np.zeros(A.n)
    r = SV.AbmcIluGmresIr(Ar.val, Ar.cind, Ar.rptr, L_.val, L_.cind, L_.rptr, U_.val, U_.cind, U_.rptr, sc, nc, 16,
                          b, x, nb, 20, 30, A.n, 1e-8)
    assert r.converged and port.relative_residual(Ar, b, x) <= 1e-8 * 1.01
    assert r.h2d_bytes > 0 and r.d2h_bytes == 8 * A.n


def test_gmres_ir_needs_mixed_system():
    A = P.poisson2d(16)
    sysm = SV.System(A, m_max=10)
    sysm.set_rhs(A.matvec(np.ones(A.n)))
    with pytest.raises(L.SenkError):
        sysm.gmres_ir(1.0, 5, 10, 1e-8)
    sysm.close()


def test_ir_only_system_solves_and_refuses_plain_solvers():
    """desc.mixed = 2 (what the drop-in GMRES-IR entry uses): no FP64
    preconditioner or basis; GMRES-IR works, the FP64 solvers refuse."""
    import numpy as np
    from senk_gb300 import lib as L
    from senk_gb300 import problems as P
    from senk_gb300 import setup as S
    from senk_gb300 import solver as SV
    A = P.convdiff3d(24, 0.5)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    Lf, Uf, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    b = Ar.matvec(P.uniform_solution(A.n, 0)[LP])
    nb = float(np.linalg.norm(b))
    sy = SV.System(Ar, Lf, Uf, L.PC_ILU_ABMC, sc, nc, 16, m_max=30, mixed=2)
    try:
        sy.set_rhs(b)
        r = sy.gmres_ir(nb, 20, 30, 1e-8)
        x = sy.get_x()
        assert r.converged and np.linalg.norm(b - Ar.matvec(x)) / nb < 1e-8
        with pytest.raises(L.SenkError):
            sy.gmres(nb, 10, 30, 1e-8)
    finally:
        sy.close()
