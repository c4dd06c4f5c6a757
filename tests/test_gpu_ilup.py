"""ILU(p) factors (include/senk_matrix.hpp:450-549, Ilup) on the GPU path, p = 1
and 2: the host Ilup factors equal the oracle's bit for bit; their level-set
sweeps (natural order; fill-in couples rows a colouring of A would separate, so
the reference's colour schedules do not apply to them) match the oracle's
sequential sweeps; IluGmresm with them gives the oracle's iteration count and
fewer iterations than ILU(0)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S
from senk_gb300 import solver as SV

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("case", ["poisson64", "convdiff16"])
@pytest.mark.parametrize("p", [1, 2])
def test_ilup_sweeps_and_gmres(port, case, p):
    import torch
    A = {"poisson64": lambda: P.poisson2d(64), "convdiff16": lambda: P.convdiff3d(16, 0.5)}[case]()
    F = S.Ilup(A, p)
    Fo = port.ilup(A, p)
    assert np.array_equal(F.rptr, Fo.rptr) and np.array_equal(F.cind, Fo.cind)
    assert np.array_equal(F.val.view(np.uint64), Fo.val.view(np.uint64))
    Lf, Uf, _ = S.Split(F, "L-DU", True)
    # plan sweeps against the oracle's sequential sweeps
    h = C.c_void_p()
    keep = [np.ascontiguousarray(a) for a in (Lf.val, Lf.cind, Lf.rptr, Uf.val, Uf.cind, Uf.rptr)]
    L.check("plan", L.lib().senk_ilu_plan_create(C.byref(h), L.F64, A.n, *[L.ptr(a) for a in keep], L.PC_ILU,
                                                 None, 0, 1))
    try:
        v = np.random.default_rng(p).uniform(-1, 1, A.n)
        xd = torch.from_numpy(v).cuda()
        yd = torch.zeros_like(xd)
        L.check("apply", L.lib().senk_ilu_plan_apply(h, xd.data_ptr(), yd.data_ptr(), None))
        L.check("status", L.lib().senk_ilu_plan_status(h, None))
        want = port.sptrsv(Uf, port.sptrsv(Lf, v, False), True)
        assert _rel(yd.cpu().numpy(), want) <= 1e-12
    finally:
        L.lib().senk_ilu_plan_destroy(h)
    # IluGmresm(30) with the ILU(p) factors against the oracle's count
    b = A.matvec(np.ones(A.n))
    nb = float(np.linalg.norm(b))
    x = np.zeros(A.n)
    r = SV.IluGmresm(A.val, A.cind, A.rptr, Lf.val, Lf.cind, Lf.rptr, Uf.val, Uf.cind, Uf.rptr, b, x, nb, 300, 30,
                     A.n, 1e-8)
    _, it, _, _ = port.solve("gmres", A, b, L=Lf, U=Uf, pc=oracle.PC_ILU, outer=300, m=30, eps=1e-8, nrm_b=nb)
    assert r.converged and abs(r.iters - it) <= 2, (r.iters, it)
    assert port.relative_residual(A, b, x) < 2e-8
    L0, U0, _ = S.Split(S.Ilu0(A), "L-DU", True)
    x0 = np.zeros(A.n)
    r0 = SV.IluGmresm(A.val, A.cind, A.rptr, L0.val, L0.cind, L0.rptr, U0.val, U0.cind, U0.rptr, b, x0, nb, 300, 30,
                      A.n, 1e-8)
    assert r.iters < r0.iters
