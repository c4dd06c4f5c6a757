"""Host checks of the synthetic workload generators."""
import numpy as np
import scipy.sparse as sp

from senk_gb300 import problems as P


def test_block27_structure_and_dominance():
    n = 5
    A = P.block27(n, seed=4)
    assert A.n == 3 * n ** 3
    M = sp.csr_matrix((A.val, A.cind, A.rptr), shape=(A.n, A.n))
    # sorted columns with the diagonal in every row; dense 3x3 blocks
    for r in range(A.n):
        c = A.cind[A.rptr[r]:A.rptr[r + 1]]
        assert np.all(np.diff(c) > 0) and r in c and len(c) % 3 == 0
    # interior node: 27 blocks
    mid = (n // 2) * (1 + n + n * n)
    assert A.rptr[3 * mid + 1] - A.rptr[3 * mid] == 81
    # block diagonal dominance 1.1: lambda_min(D_i) >= 1.1 * sum ||A_ij||_2
    D = M.toarray()
    for node in (0, mid, n ** 3 - 1):
        rows = slice(3 * node, 3 * node + 3)
        lam = np.linalg.eigvalsh(D[rows, rows]).min()
        off = 0.0
        for nb in set(A.cind[A.rptr[3 * node]:A.rptr[3 * node + 1]] // 3) - {node}:
            off += np.linalg.norm(D[rows, 3 * nb:3 * nb + 3], 2)
        assert lam >= 1.1 * off - 1e-12
    assert np.array_equal(P.block27(n, seed=4).val, A.val)  # seeded


def test_node_permutation_expansion_and_graph():
    A = P.block27(3, seed=0)
    G = P.node_graph(A)
    assert G.n == 27 and G.nnz == int(np.sum(np.diff(A.rptr)) // 9)
    LPn = np.random.default_rng(0).permutation(27)
    LP, RP = P.expand_node_permutation(LPn)
    assert np.array_equal(LP[RP], np.arange(81)) and np.array_equal(LP[3 * 5 + 2], 3 * LPn[5] + 2)
