"""Host setup of the benchmarked systems at their full sizes against the oracle.

The small-case tests (test_setup_parity.py) pin every setup routine bit for bit;
these repeat the check on the exact systems the timed solves run on, so that the
GPU solves there start from arrays identical to the oracle's:

- convdiff3d 128^3 (Pe 0.5), ABMC bsize 16 connect, ILU(0), L-DU split with the
  inverted diagonal: size_color, LP, RP, the reordered matrix, both factors and
  the right-hand side compared with memcmp;
- vardiff3d 160^3 (contrast 8, seed 0), same pipeline;
- block27 with 3x3 node blocks, node-graph ABMC bsize 4, block-zero pattern,
  ILU(0), BCSR conversion of both factors.  At 96^3 this system holds 215 M
  nonzeros (several GB per copy), more than a CPU test should build; it runs at
  48^3 (26 M nonzeros), which exercises the same code on every row shape.

Each case takes a few seconds per side.
"""
import numpy as np
import pytest

from senk_gb300 import problems as P
from senk_gb300 import setup as S


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes()


def same_csr(a, b):
    return a.n == b.n and same(a.rptr, b.rptr) and same(a.cind, b.cind) and same(a.val, b.val)


@pytest.mark.slow
@pytest.mark.parametrize("case", ["convdiff128", "vardiff160"])
def test_scalar_setup_matches_oracle_full_size(port, case):
    if case == "convdiff128":
        A, xt = P.convdiff3d(128, 0.5), P.uniform_solution(128 ** 3, 0)
    else:
        A = P.vardiff3d(160, 1.5, 8.0, 0)
        xt = P.normal_solution(A.n, 1)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    onc, osc, oLP, oRP = port.abmc_permutation(A.cind, A.rptr, A.n, 16, False, "connect")
    assert nc == onc and same(sc, osc) and same(LP, oLP) and same(RP, oRP)
    Ar, Ao = S.Reordering(A, LP, RP), port.reordering(A, oLP, oRP)
    assert same_csr(Ar, Ao)
    F, Fo = S.Ilu0(Ar), port.ilu0(Ao)
    assert same(F.val, Fo.val)
    L, U, _ = S.Split(F, "L-DU", True)
    oL, oU, _ = port.split(Fo, "L-DU", True)
    assert same_csr(L, oL) and same_csr(U, oU)
    assert same(Ar.matvec(xt[LP]), Ao.matvec(xt[oLP]))


@pytest.mark.slow
def test_block_setup_matches_oracle(port):
    n = 48
    A, G = P.block27(n, seed=0), P.block27_node_graph(n)
    nc, sc, LPn, RPn = S.GetABMCPermutation(G.cind, G.rptr, G.n, 4, False, "connect")
    onc, osc, oLPn, oRPn = port.abmc_permutation(G.cind, G.rptr, G.n, 4, False, "connect")
    assert nc == onc and same(sc, osc) and same(LPn, oLPn) and same(RPn, oRPn)
    LP, RP = P.expand_node_permutation(LPn, 3)
    Ar, Ao = S.Reordering(A, LP, RP), port.reordering(A, LP, RP)
    assert same_csr(Ar, Ao)
    Z, Zo = S.AllocBlockZero(Ar, 3, 3), port.alloc_block_zero(Ao, 3, 3)
    assert same_csr(Z, Zo)
    F, Fo = S.Ilu0(Z), port.ilu0(Zo)
    assert same(F.val, Fo.val)
    L, U, _ = S.Split(F, "L-DU", True)
    oL, oU, _ = port.split(Fo, "L-DU", True)
    assert same_csr(L, oL) and same_csr(U, oU)
    for f, fo in ((L, oL), (U, oU)):
        assert all(same(x, y) for x, y in zip(S.Csr2Bcsr(f, 3, 3), port.csr2bcsr(fo, 3, 3)))
