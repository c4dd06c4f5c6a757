"""Host setup of the product (include/senk_matrix.hpp, include/senk_graph.hpp,
through the C ABI) against the oracle: integer arrays bit-identical, ILU values
to 0 ULP (same operations in the same order)."""
import numpy as np
import pytest

from senk_gb300 import problems as P
from senk_gb300 import setup as S


CASES = {
    "poisson128": lambda: P.poisson2d(128),
    "convdiff16": lambda: P.convdiff3d(16, 0.5),
    "convdiff24": lambda: P.convdiff3d(24, 0.5),
    "vardiff16": lambda: P.vardiff3d(16, 1.5, 4.0, 3),
}


def eq(a, b):
    return a.dtype == b.dtype and np.array_equal(a, b)


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("bsize,method", [(16, "connect"), (8, "simple"), (32, "connect"), (1, "connect")])
def test_abmc_matches_oracle(port, case, bsize, method):
    A = CASES[case]()
    if A.n % bsize:
        pytest.skip("N not a multiple of bsize")
    a = S.GetABMCPermutation(A.cind, A.rptr, A.n, bsize, False, method)
    o = port.abmc_permutation(A.cind, A.rptr, A.n, bsize, False, method)
    assert a[0] == o[0] and all(eq(x, y) for x, y in zip(a[1:], o[1:]))


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("sym", [False, True])
def test_amc_matches_oracle(port, case, sym):
    A = CASES[case]()
    a = S.GetAMCPermutation(A.cind, A.rptr, A.n, sym)
    o = port.amc_permutation(A.cind, A.rptr, A.n, sym)
    assert a[0] == o[0] and all(eq(x, y) for x, y in zip(a[1:], o[1:]))


@pytest.mark.parametrize("case", sorted(CASES))
def test_reorder_ilu0_split_match_oracle(port, case):
    A = CASES[case]()
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, A.n, 16, False, "connect") if A.n % 16 == 0 else \
        port.amc_permutation(A.cind, A.rptr, A.n, False)
    Ar, Ao = S.Reordering(A, LP, RP), port.reordering(A, LP, RP)
    assert eq(Ar.val, Ao.val) and eq(Ar.cind, Ao.cind) and eq(Ar.rptr, Ao.rptr)
    F, Fo = S.Ilu0(Ar), port.ilu0(Ao)
    assert eq(F.val, Fo.val)
    for key in ("L-DU", "LD-U", "L-D-U", "LU-D"):
        for inv in (True, False):
            got, want = S.Split(F, key, inv), port.split(Fo, key, inv)
            for g, w in zip(got, want):
                assert (g is None) == (w is None), key
                if g is None:
                    continue
                if hasattr(g, "val"):
                    assert eq(g.val, w.val) and eq(g.cind, w.cind) and eq(g.rptr, w.rptr), key
                else:
                    assert eq(g, w), key


@pytest.mark.parametrize("p", [0, 1, 2, 3])
def test_ilup_and_level_zero_match_oracle(port, p):
    A = P.convdiff3d(12, 0.5)
    for ours, theirs in ((S.Ilup, port.ilup), (S.AllocLevelZero, port.alloc_level_zero)):
        a, o = ours(A, p), theirs(A, p)
        assert eq(a.rptr, o.rptr) and eq(a.cind, o.cind) and eq(a.val, o.val)


@pytest.mark.parametrize("bnl,bnw", [(8, 1), (2, 2), (4, 1), (2, 1), (4, 2)])
def test_block_patterns_match_oracle(port, bnl, bnw):
    A = P.poisson2d(32)
    a, o = S.AllocBlockZero(A, bnl, bnw), port.alloc_block_zero(A, bnl, bnw)
    assert eq(a.rptr, o.rptr) and eq(a.cind, o.cind) and eq(a.val, o.val)
    ba, bo = S.Csr2Bcsr(A, bnl, bnw), port.csr2bcsr(A, bnl, bnw)
    assert all(eq(x, y) for x, y in zip(ba, bo))


def test_ilu_p_factor_through_level_zero_and_ilu0(port):
    # ILU(p) values: pattern from AllocLevelZero, then ILU(0) on that pattern.
    A = P.convdiff3d(10, 0.5)
    pat = S.AllocLevelZero(A, 1)
    a, o = S.Ilu0(pat), port.ilu0(port.alloc_level_zero(A, 1))
    assert eq(a.val, o.val)


def test_golden_c1_setup(golden):
    import hashlib
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    A = P.poisson2d(128)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    g = golden["c1"]["abmc16"]
    assert nc == g["num_color"] and sc.tolist() == g["size_color"] and sha(LP) == g["LP_sha"]
    Ar = S.Reordering(A, LP, RP)
    L, U, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    assert sha(L.val) == g["L_sha"] and sha(U.val) == g["U_sha"]


@pytest.mark.parametrize("bnl,bnw", [(1, 1), (2, 1), (2, 2), (3, 3), (4, 1), (4, 2), (8, 1), (8, 2)])
def test_csr2bcsr_of_factors_matches_oracle(port, bnl, bnw):
    # L rows without lower entries (row 0, and the first rows of ABMC blocks)
    # take the next row's first entry, as in the reference
    A = P.convdiff3d(12, 0.5)
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, A.n, 16, False, "connect")
    L, U, _ = S.Split(S.Ilu0(S.Reordering(A, LP, RP)), "L-DU", True)
    assert np.count_nonzero(np.diff(L.rptr) == 0) > 1
    for F in (L, U):
        a, o = S.Csr2Bcsr(F, bnl, bnw), port.csr2bcsr(F, bnl, bnw)
        assert all(eq(x, y) for x, y in zip(a, o))
    assert S.Csr2Bcsr(L, bnl, bnw)[0][0] != 0.0


def test_csr2bcsr_of_factors_matches_reference(port, ref):
    A = P.convdiff3d(8, 0.5)
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, A.n, 8, False, "connect")
    L, U, _ = S.Split(S.Ilu0(S.Reordering(A, LP, RP)), "L-DU", True)
    for bnl, bnw in ((8, 1), (2, 2), (4, 2)):
        for F in (L, U):
            a, r = S.Csr2Bcsr(F, bnl, bnw), ref.csr2bcsr(F, bnl, bnw)
            assert all(eq(x, y) for x, y in zip(a, r))
