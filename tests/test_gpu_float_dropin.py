"""T = float instantiations of the drop-in solvers (Gmresm, AmcIluGmresm, Gcrm,
IluGcrm, Bicgstab, IluBicgstab) on the 2D Poisson problem: each converges to its
FP32 tolerance, and the FP64 true residual of the FP32 solution is checked."""
import numpy as np
import pytest

from senk_gb300 import problems as P
from senk_gb300 import setup as S
from senk_gb300 import solver as SV

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sys32():
    A = P.poisson2d(64)
    b = A.matvec(np.ones(A.n))
    Lf, Uf, _ = S.Split(S.Ilu0(A), "L-DU", True)
    nc, sc, LP, RP = S.GetAMCPermutation(A.cind, A.rptr, A.n, False)
    Ar = S.Reordering(A, LP, RP)
    La, Ua, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    return A, b, Lf, Uf, Ar, La, Ua, sc, nc, LP


def _true(A, b, x):
    return float(np.linalg.norm(b - A.matvec(x.astype(np.float64))) / np.linalg.norm(b))


def test_float_solvers(sys32):
    A, b, Lf, Uf, Ar, La, Ua, sc, nc, LP = sys32
    f = np.float32
    nb = float(np.linalg.norm(b))
    b32 = b.astype(f)
    runs = {
        "Gmresm": lambda x: SV.Gmresm(A.val, A.cind, A.rptr, b32, x, nb, 200, 30, A.n, 1e-5),
        "Gcrm": lambda x: SV.Gcrm(A.val, A.cind, A.rptr, b32, x, nb, 400, 20, A.n, 1e-5),
        "Bicgstab": lambda x: SV.Bicgstab(A.val, A.cind, A.rptr, b32, x, nb, 5000, A.n, 1e-5),
        "IluGcrm": lambda x: SV.IluGcrm(A.val, A.cind, A.rptr, Lf.val, Lf.cind, Lf.rptr, Uf.val, Uf.cind, Uf.rptr,
                                        b32, x, nb, 400, 20, A.n, 1e-5),
        "IluBicgstab": lambda x: SV.IluBicgstab(A.val, A.cind, A.rptr, Lf.val, Lf.cind, Lf.rptr, Uf.val, Uf.cind,
                                                Uf.rptr, b32, x, nb, 5000, A.n, 1e-5),
    }
    for name, run in runs.items():
        x = np.zeros(A.n, f)
        r = run(x)
        assert r.converged, name
        assert _true(A, b, x) < 1e-4, (name, _true(A, b, x))
    x = np.zeros(A.n, f)
    br = b[LP].astype(f)
    r = SV.AmcIluGmresm(Ar.val, Ar.cind, Ar.rptr, La.val, La.cind, La.rptr, Ua.val, Ua.cind, Ua.rptr, sc, nc, br, x,
                        nb, 200, 30, A.n, 1e-5)
    assert r.converged and _true(Ar, b[LP], x) < 1e-4
