"""The device ABMC ordering's algorithm (tests/abmc_emulate.py, a step-for-step
CPU restatement of senk_gb300/csrc/colour.cu: colours by parallel rounds)
gives exactly the reference's GetABMCPermutation with simple blocking and, for
bs = 1, GetAMCPermutation (the product's host restatement, pinned to the
reference); the orderings are valid (colours independent, LP and RP inverse
permutations keeping blocks whole)."""
import numpy as np
import pytest

import abmc_emulate as E
from senk_gb300 import problems as P
from senk_gb300 import setup as S

CASES = {
    "poisson64": lambda: P.poisson2d(64),
    "convdiff16": lambda: P.convdiff3d(16, 0.5),
    "vardiff12": lambda: P.vardiff3d(12, 1.5, 4.0, 3),
    "block27_4": lambda: P.block27(4, seed=0),
}


def _shuffled(A, seed):
    """A symmetrically permuted at random: no longer a grid in index order."""
    p = np.random.default_rng(seed).permutation(A.n).astype(np.int32)
    rp = np.empty_like(p)
    rp[p] = np.arange(A.n, dtype=np.int32)
    return S.Reordering(A, p, rp)


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("bs", [1, 4, 16])
@pytest.mark.parametrize("shuffle", [False, True])
def test_emulated_ordering_equals_the_reference(case, bs, shuffle):
    A = CASES[case]()
    if A.n % bs:
        pytest.skip("N not a multiple of bs")
    if shuffle:
        A = _shuffled(A, bs)
    nc, sc, LP, RP, rounds = E.abmc(A.cind, A.rptr, A.n, bs)
    E.check_ordering(A.cind, A.rptr, A.n, bs, nc, sc, LP, RP)
    rnc, rsc, rLP, rRP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bs, False, "simple")
    assert nc == rnc and np.array_equal(sc, rsc) and np.array_equal(LP, rLP) and np.array_equal(RP, rRP)
    if bs == 1:
        anc, asc, aLP, aRP = S.GetAMCPermutation(A.cind, A.rptr, A.n, False)
        assert nc == anc and np.array_equal(sc, asc) and np.array_equal(LP, aLP)
    print(f"{case} bs {bs} shuffled {shuffle}: {nc} colours, {rounds} rounds")
