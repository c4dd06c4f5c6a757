"""The drop-in entries keep their device systems between calls: a second call
with the same arrays uploads only b and x and gives the same answer; a matrix
changed in place (same addresses, new values) is rebuilt; with the cache off
every call uploads everything."""
import numpy as np
import pytest

from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S
from senk_gb300 import solver as SV

pytestmark = pytest.mark.gpu


def _system(scale=1.0):
    A = P.convdiff3d(24, 0.5)
    A.val *= scale
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    Lf, Uf, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    return Ar, Lf, Uf, sc, nc


def _solve(Ar, Lf, Uf, sc, nc, b):
    x = np.zeros(Ar.n)
    r = SV.AbmcIluGmresm(Ar.val, Ar.cind, Ar.rptr, Lf.val, Lf.cind, Lf.rptr, Uf.val, Uf.cind, Uf.rptr, sc, nc, 16,
                         b, x, float(np.linalg.norm(b)), 100, 30, Ar.n, 1e-8)
    return r, x


def test_second_call_reuses_the_system_and_a_changed_matrix_is_rebuilt():
    L.lib().senk_dropin_cache(1)
    Ar, Lf, Uf, sc, nc = _system()
    b = Ar.matvec(np.random.default_rng(1).uniform(-1, 1, Ar.n))
    r1, x1 = _solve(Ar, Lf, Uf, sc, nc, b)
    r2, x2 = _solve(Ar, Lf, Uf, sc, nc, b)
    assert r1.converged and r2.converged and r1.iters == r2.iters
    assert np.array_equal(x1, x2)
    assert r1.h2d_bytes > 10 * 16 * Ar.n and r2.h2d_bytes == 2 * 8 * Ar.n
    # new values in the same arrays: A doubled, factors of the doubled matrix
    A2, L2, U2, _, _ = _system(2.0)
    Ar.val[:] = A2.val
    Lf.val[:] = L2.val
    Uf.val[:] = U2.val
    r3, x3 = _solve(Ar, Lf, Uf, sc, nc, b)
    assert r3.converged and r3.h2d_bytes > 10 * 16 * Ar.n
    assert np.linalg.norm(b - Ar.matvec(x3)) / np.linalg.norm(b) < 2e-8
    assert np.allclose(x3, 0.5 * x1, rtol=0, atol=1e-6 * np.abs(x1).max())


def test_cache_off_uploads_every_call():
    prev = L.lib().senk_dropin_cache(0)
    try:
        Ar, Lf, Uf, sc, nc = _system()
        b = Ar.matvec(np.ones(Ar.n))
        r1, _ = _solve(Ar, Lf, Uf, sc, nc, b)
        r2, _ = _solve(Ar, Lf, Uf, sc, nc, b)
        assert r1.h2d_bytes == r2.h2d_bytes > 10 * 16 * Ar.n
    finally:
        L.lib().senk_dropin_cache(prev)
