"""The measurement plan's larger workloads on the GPU, at parity-test sizes and
at 64^3, against the oracle:

* variable-coefficient diffusion (the 160^3 workload's family): plain FP64
  ABMC-ILU(0)-GMRES(50) against the oracle's iteration count, and FP64-outer
  GMRES-IR with FP32 factors, sweeps and inner SpMV, both to 1e-10 FP64 true
  residual; the mixed solution's distance from the plain one is checked;
* the block-3x3 27-point system (the 96^3 workload's family): ILUB(3x3) with
  ABMC colouring of the node graph, FP64 and FP32 sweeps against the oracle's
  sequential BCSR sweeps on the same reordered system, GCR(20) to 1e-8 against
  the oracle's count, and FP64-outer GCR-IR with FP32 ILUB and inner SpMV."""
import numpy as np
import pytest

import oracle
from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S
from senk_gb300 import solver as SV

pytestmark = pytest.mark.gpu


def test_vardiff_gmres50_plain_and_mixed_to_1e10(port):
    A = P.vardiff3d(24, 1.5, 8.0, 0)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    Lf, Uf, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    b = Ar.matvec(P.normal_solution(A.n, 1)[LP])
    nb = float(np.linalg.norm(b))
    _, it, _, _ = port.solve("gmres", Ar, b, L=Lf, U=Uf, pc=oracle.PC_ILU_ABMC, cptr=sc, cnum=nc, bsize=16,
                             outer=10000 // 50, m=50, eps=1e-10, nrm_b=nb)
    sy = SV.System(Ar, Lf, Uf, L.PC_ILU_ABMC, sc, nc, 16, m_max=50, mixed=1)
    try:
        sy.set_rhs(b)
        r = sy.gmres(nb, 10000 // 50, 50, 1e-10)
        xp = sy.get_x()
        assert r.converged and abs(r.iters - it) <= 2
        assert np.linalg.norm(b - Ar.matvec(xp)) / nb < 2e-10
        sy.set_rhs(b)
        ri = sy.gmres_ir(nb, 30, 50, 1e-10)
        xm = sy.get_x()
        assert ri.converged and np.linalg.norm(b - Ar.matvec(xm)) / nb <= 1e-10
        # the mixed solution is as close to the plain one as the tolerance allows
        assert np.linalg.norm(xm - xp) / np.linalg.norm(xp) < 1e-7
    finally:
        sy.close()


def _block27_abmc(n=6, node_bsize=4):
    A = P.block27(n, seed=1)
    G = P.block27_node_graph(n)
    nc, sc, LPn, _ = S.GetABMCPermutation(G.cind, G.rptr, G.n, node_bsize, False, "connect")
    LP, RP = P.expand_node_permutation(LPn, 3)
    Ar = S.Reordering(A, LP, RP)
    Lf, Uf, _ = S.Split(S.Ilu0(S.AllocBlockZero(Ar, 3, 3)), "L-DU", True)
    return Ar, S.Csr2Bcsr(Lf, 3, 3), S.Csr2Bcsr(Uf, 3, 3), sc, nc, 3 * node_bsize, LP


def test_block27_ilub_abmc_gcr20(port):
    Ar, bl, bu, sc, nc, bs, LP = _block27_abmc()
    b = Ar.matvec(P.uniform_solution(Ar.n, 2)[LP])
    nb = float(np.linalg.norm(b))
    _, it, _, _ = port.solve("gcr", Ar, b, L=bl, U=bu, pc=oracle.PC_ILUB_ABMC, cptr=sc, cnum=nc, bsize=bs, bnl=3,
                             bnw=3, outer=500, m=20, eps=1e-8, nrm_b=nb)
    sy = SV.System(Ar, bl, bu, L.PC_ILUB_ABMC, sc, nc, bs, m_max=0, block=(3, 3))
    try:
        sy.set_rhs(b)
        r = sy.gcr(nb, 500, 20, 1e-8)
        x = sy.get_x()
        assert r.converged and abs(r.iters - it) <= 20
        assert np.linalg.norm(b - Ar.matvec(x)) / nb < 1e-8
    finally:
        sy.close()


def _vardiff_case(n, seed=0):
    A = P.vardiff3d(n, 1.5, 8.0, seed)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    Lf, Uf, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    b = Ar.matvec(P.normal_solution(A.n, 1)[LP])
    return Ar, Lf, Uf, sc, nc, b


def test_vardiff64_gmres50_plain_and_mixed_to_1e10():
    """64^3 (262,144 rows): GPU GMRES(50) within 2 iterations of the oracle's
    (run with all host threads), GMRES-IR to 1e-10, and the mixed solution's
    relative distance from the plain one."""
    import os
    Ar, Lf, Uf, sc, nc, b = _vardiff_case(64)
    nb = float(np.linalg.norm(b))
    port = oracle.port(threads=os.cpu_count() or 1)
    _, it, _, _ = port.solve("gmres", Ar, b, L=Lf, U=Uf, pc=oracle.PC_ILU_ABMC, cptr=sc, cnum=nc, bsize=16,
                             outer=10000 // 50, m=50, eps=1e-10, nrm_b=nb)
    port.set_threads(1)
    sy = SV.System(Ar, Lf, Uf, L.PC_ILU_ABMC, sc, nc, 16, m_max=50, mixed=1)
    try:
        sy.set_rhs(b)
        r = sy.gmres(nb, 10000 // 50, 50, 1e-10)
        xp = sy.get_x()
        assert r.converged and abs(r.iters - it) <= 2, (r.iters, it)
        assert np.linalg.norm(b - Ar.matvec(xp)) / nb < 2e-10
        sy.set_rhs(b)
        ri = sy.gmres_ir(nb, 30, 50, 1e-10)
        xm = sy.get_x()
        assert ri.converged and np.linalg.norm(b - Ar.matvec(xm)) / nb <= 1e-10
        assert np.linalg.norm(xm - xp) / np.linalg.norm(xp) < 1e-7
    finally:
        sy.close()


@pytest.mark.parametrize("n", [6, 16])
def test_block27_ilub_sweeps_f64_and_f32(port, n):
    """ILUB(3x3) application on the GPU, FP64 and FP32 factors, against the
    oracle's ABMC BCSR sweeps in the same precision."""
    Ar, bl, bu, sc, nc, bs, LP = _block27_abmc(n)
    v = np.random.default_rng(4).uniform(-1, 1, Ar.n)
    for T, tol in ((np.float64, 1e-12), (np.float32, 1e-5)):
        sy = SV.System(Ar, (bl[0].astype(T), bl[1], bl[2]), (bu[0].astype(T), bu[1], bu[2]), L.PC_ILUB_ABMC, sc,
                       nc, bs, dtype=T, m_max=1, block=(3, 3))
        try:
            got = sy.apply_precond(v.astype(T))
        finally:
            sy.close()
        want = port.ilub_apply(bl, bu, v, 3, 3, sc, nc, bs, dtype=T)
        assert np.max(np.abs(got - want)) <= tol * np.max(np.abs(want))


def test_block27_64_gcr20_plain_and_mixed():
    """64^3 nodes (786,432 rows, about 62M entries): ILUB(3x3)-GCR(20) in FP64
    within one restart of the oracle's count, and GCR-IR (FP32 inner GCR(20),
    FP32 ILUB and SpMV) to the same 1e-8 FP64 true residual."""
    import os
    Ar, bl, bu, sc, nc, bs, LP = _block27_abmc(64)
    b = Ar.matvec(P.uniform_solution(Ar.n, 2)[LP])
    nb = float(np.linalg.norm(b))
    port = oracle.port(threads=os.cpu_count() or 1)
    _, it, _, _ = port.solve("gcr", Ar, b, L=bl, U=bu, pc=oracle.PC_ILUB_ABMC, cptr=sc, cnum=nc, bsize=bs, bnl=3,
                             bnw=3, outer=500, m=20, eps=1e-8, nrm_b=nb)
    port.set_threads(1)
    sy = SV.System(Ar, bl, bu, L.PC_ILUB_ABMC, sc, nc, bs, m_max=0, block=(3, 3), mixed=1)
    try:
        sy.set_rhs(b)
        r = sy.gcr(nb, 500, 20, 1e-8)
        xp = sy.get_x()
        assert r.converged and abs(r.iters - it) <= 20, (r.iters, it)
        assert np.linalg.norm(b - Ar.matvec(xp)) / nb < 1e-8
        sy.set_rhs(b)
        ri = sy.gcr_ir(nb, 30, 20, 1e-8)
        xm = sy.get_x()
        assert ri.converged and np.linalg.norm(b - Ar.matvec(xm)) / nb <= 1e-8
        assert np.linalg.norm(xm - xp) / np.linalg.norm(xp) < 1e-5
    finally:
        sy.close()
