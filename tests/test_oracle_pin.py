"""Pins the oracle (the C restatement) to the reference.

* against the golden fixtures the reference produced (tests/golden/, made by
  tests/golden/make_golden.py): runs on every machine;
* against the reference itself, compiled from its own headers into oracle/_ref:
  runs only where the reference sources exist.
"""
import hashlib

import numpy as np
import pytest

import oracle
from senk_gb300 import problems as P


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def c1():
    A = P.poisson2d(128)
    b = A.matvec(np.ones(A.n))
    return A, b


def test_c1_sizes(c1, golden):
    A, _ = c1
    assert (A.n, A.nnz) == (golden["c1"]["N"], golden["c1"]["nnz"]) == (16384, 81408)


def test_c1_natural_ilu_matches_golden(port, c1, golden):
    A, b = c1
    L, U, _ = port.split(port.ilu0(A), "L-DU", True)
    g = golden["c1"]["ilu_natural"]
    assert sha(L.val) == g["L_sha"] and sha(U.val) == g["U_sha"]
    assert sha(np.concatenate([L.rptr, L.cind])) == g["Lpat_sha"]
    assert sha(np.concatenate([U.rptr, U.cind])) == g["Upat_sha"]


@pytest.mark.parametrize("method,pc,key,m", [
    ("gmres", oracle.PC_ILU, "IluGmresm_m30", 30),
    ("bicgstab", oracle.PC_ILU, "IluBicgstab", 0),
    ("gcr", oracle.PC_ILU, "IluGcrm_m20", 20),
    ("bicgstab", oracle.PC_NONE, "Bicgstab", 0),
])
def test_c1_solvers_match_golden(port, c1, golden, method, pc, key, m):
    A, b = c1
    L, U, _ = port.split(port.ilu0(A), "L-DU", True)
    kw = dict(outer=10000 // m, m=m) if m else dict(max_iter=10000)
    x, it, res, conv = port.solve(method, A, b, L=L, U=U, pc=pc, eps=1e-8, **kw)
    g = golden["c1"][key]
    assert it == g["iters"]
    assert float("%e" % res) == pytest.approx(g["res"], rel=1e-6)


def test_c1_unpreconditioned_gmres_matches_golden(port, c1, golden):
    A, b = c1
    _, it, res, _ = port.solve("gmres", A, b, pc=oracle.PC_NONE, outer=10000 // 30, m=30, eps=1e-8)
    assert it == golden["c1"]["Gmresm_m30"]["iters"]


def test_c1_abmc_and_amc_match_golden(port, c1, golden):
    A, b = c1
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, A.n, 16, False, "connect")
    g = golden["c1"]["abmc16"]
    assert nc == g["num_color"] and sc.tolist() == g["size_color"]
    assert sha(LP) == g["LP_sha"] and sha(RP) == g["RP_sha"]
    Ar = port.reordering(A, LP, RP)
    assert sha(np.concatenate([Ar.rptr, Ar.cind])) == g["A_sha"] and sha(Ar.val) == g["Aval_sha"]
    L, U, _ = port.split(port.ilu0(Ar), "L-DU", True)
    assert sha(L.val) == g["L_sha"] and sha(U.val) == g["U_sha"]
    _, it, res, _ = port.solve("gmres", Ar, b[LP], L=L, U=U, pc=oracle.PC_ILU_ABMC, cptr=sc, cnum=nc,
                               bsize=16, outer=10000 // 30, m=30, eps=1e-8, nrm_b=float(np.linalg.norm(b)))
    assert it == golden["c1"]["AbmcIluGmresm_m30"]["iters"]
    nc2, sc2, LP2, _ = port.amc_permutation(A.cind, A.rptr, A.n, False)
    assert nc2 == golden["c1"]["amc"]["num_color"] and sha(LP2) == golden["c1"]["amc"]["LP_sha"]


def test_c1_ilub_matches_golden(port, c1, golden):
    A, b = c1
    Ab = port.alloc_block_zero(A, 8, 1)
    g = golden["c1"]["ilub_8x1"]
    assert Ab.nnz == g["nnz"] and sha(np.concatenate([Ab.rptr, Ab.cind])) == g["pattern_sha"]
    L, U, _ = port.split(port.ilu0(Ab), "L-DU", True)
    bl, bu = port.csr2bcsr(L, 8, 1), port.csr2bcsr(U, 8, 1)
    assert sha(bl[0]) == g["Lb_sha"] and sha(bu[0]) == g["Ub_sha"]
    _, it, _, _ = port.solve("gmres", A, b, L=bl, U=bu, pc=oracle.PC_ILUB, bnl=8, bnw=1,
                             outer=10000 // 30, m=30, eps=1e-8)
    assert it == golden["c1"]["IlubGmresm_8x1_m30"]["iters"]


def test_c1_ilub_gcr_bicgstab_and_2x2_match_golden(port, c1, golden):
    A, b = c1
    L, U, _ = port.split(port.ilu0(port.alloc_block_zero(A, 8, 1)), "L-DU", True)
    bl, bu = port.csr2bcsr(L, 8, 1), port.csr2bcsr(U, 8, 1)
    _, it, _, _ = port.solve("gcr", A, b, L=bl, U=bu, pc=oracle.PC_ILUB, bnl=8, bnw=1, outer=10000 // 20, m=20,
                             eps=1e-8)
    assert it == golden["c1"]["IlubGcrm_8x1_m20"]["iters"]
    _, it, _, _ = port.solve("bicgstab", A, b, L=bl, U=bu, pc=oracle.PC_ILUB, bnl=8, bnw=1, max_iter=10000,
                             eps=1e-8)
    assert it == golden["c1"]["IlubBicgstab_8x1"]["iters"]
    L2, U2, _ = port.split(port.ilu0(port.alloc_block_zero(A, 2, 2)), "L-DU", True)
    _, it, _, _ = port.solve("gmres", A, b, L=port.csr2bcsr(L2, 2, 2), U=port.csr2bcsr(U2, 2, 2),
                             pc=oracle.PC_ILUB, bnl=2, bnw=2, outer=10000 // 30, m=30, eps=1e-8)
    assert it == golden["c1"]["IlubGmresm_2x2_m30"]["iters"]


def test_c1_abmc_ilub_matches_golden(port, c1, golden):
    A, b = c1
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = port.reordering(A, LP, RP)
    L, U, _ = port.split(port.ilu0(port.alloc_block_zero(Ar, 8, 1)), "L-DU", True)
    _, it, _, _ = port.solve("gmres", Ar, b[LP], L=port.csr2bcsr(L, 8, 1), U=port.csr2bcsr(U, 8, 1),
                             pc=oracle.PC_ILUB_ABMC, cptr=sc, cnum=nc, bsize=16, bnl=8, bnw=1, outer=10000 // 30,
                             m=30, eps=1e-8, nrm_b=float(np.linalg.norm(b)))
    assert it == golden["c1"]["AbmcIlubGmresm_8x1_m30"]["iters"]


def test_c1_block_jacobi_matches_golden(port, c1, golden):
    A, b = c1
    Aj = port.remove_off_diagonal(A, 16)
    g = golden["c1"]["bj16"]
    assert Aj.nnz == g["nnz"] and sha(np.concatenate([Aj.rptr, Aj.cind])) == g["pattern_sha"]
    L, U, _ = port.split(port.ilu0(Aj), "L-DU", True)
    _, it, _, _ = port.solve("gmres", A, b, L=L, U=U, pc=oracle.PC_ILU_BJ, bnum=16, outer=10000 // 30, m=30,
                             eps=1e-8)
    assert it == golden["c1"]["BjIluGmresm_16_m30"]["iters"]


def test_c1_unpreconditioned_gcr_and_bcsr_gmres_match_golden(port, c1, golden):
    A, b = c1
    _, it, _, _ = port.solve("gcr", A, b, pc=oracle.PC_NONE, outer=10000 // 20, m=20, eps=1e-8)
    assert it == golden["c1"]["Gcrm_m20"]["iters"]
    _, it, _, _ = port.solve("gmres", port.csr2bcsr(A, 2, 2), b, pc=oracle.PC_NONE, op=oracle.OP_BCSR, bnl=2,
                             bnw=2, outer=10000 // 30, m=30, eps=1e-8)
    assert it == golden["c1"]["BcsrGmresm_2x2_m30"]["iters"]


def test_c1_float_gmres_matches_golden(port, c1, golden):
    A, b = c1
    L, U, _ = port.split(port.ilu0(A), "L-DU", True)
    _, it, _, _ = port.solve("gmres", A.astype(np.float32), b, L=L, U=U, pc=oracle.PC_ILU,
                             outer=10000 // 30, m=30, eps=1e-6, dtype=np.float32,
                             nrm_b=float(np.float32(np.sqrt(np.dot(b, b)))))
    assert it == golden["c1"]["IluGmresm_float_m30"]["iters"]


def test_small_arrays_match_golden(port, small, golden):
    s = small
    A = P.Csr(s["A_val"], s["A_cind"], s["A_rptr"])
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, A.n, 16, False, "connect")
    assert np.array_equal(LP, s["LP"]) and np.array_equal(RP, s["RP"]) and np.array_equal(sc, s["size_color"])
    Ar = port.reordering(A, LP, RP)
    assert np.array_equal(Ar.val, s["Ar_val"]) and np.array_equal(Ar.cind, s["Ar_cind"])
    L, U, _ = port.split(port.ilu0(Ar), "L-DU", True)
    for k, v in dict(L_val=L.val, L_cind=L.cind, L_rptr=L.rptr, U_val=U.val, U_cind=U.cind, U_rptr=U.rptr).items():
        assert np.array_equal(v, s[k]), k
    assert np.array_equal(port.spmv_csr(Ar, s["v"]), s["y_spmv"])
    assert np.array_equal(port.ilu_apply(L, U, s["v"], sc, nc, 16), s["y_ilu_abmc"])
    assert np.array_equal(port.ilu_apply(L, U, s["v"]), s["y_ilu_seq"])
    x, it, _, _ = port.solve("gmres", Ar, s["b"], L=L, U=U, pc=oracle.PC_ILU_ABMC, cptr=sc, cnum=nc,
                             bsize=16, outer=100, m=30, eps=1e-8)
    assert it == golden["convdiff16"]["AbmcIluGmresm_m30"]["iters"]
    np.testing.assert_allclose(x, s["x_gmres"], rtol=0, atol=1e-12)


def test_generators_are_seeded():
    a, b = P.uniform_solution(1000, 0), P.uniform_solution(1000, 0)
    assert np.array_equal(a, b)
    g = P.gaussian_random_field(16, 1.5, 4.0, 3)
    assert abs(g.std() - 1.5) < 1e-12 and abs(g.mean()) < 1e-12
    A = P.vardiff3d(8, 1.0, 2.0, 1)
    assert A.n == 512 and A.nnz == 512 * 7 - 6 * 64
    d = A.val[np.concatenate([np.where(A.cind[A.rptr[i]:A.rptr[i + 1]] == i)[0] + A.rptr[i] for i in range(A.n)])]
    off = np.abs(A.matvec(np.ones(A.n)))  # row sums >= 0: weakly diagonally dominant
    assert np.all(d > 0) and np.all(off >= -1e-12)


# --------------------------------------------------- live pins vs the reference

def _vs_ref_case():
    A = P.convdiff3d(24, 0.5)
    return A


def test_live_setup_matches_reference(port, ref):
    A = _vs_ref_case()
    for bs, meth in [(16, "connect"), (8, "simple"), (32, "connect")]:
        a = port.abmc_permutation(A.cind, A.rptr, A.n, bs, False, meth)
        r = ref.abmc_permutation(A.cind, A.rptr, A.n, bs, False, meth)
        assert a[0] == r[0] and all(np.array_equal(x, y) for x, y in zip(a[1:], r[1:]))
    a = port.amc_permutation(A.cind, A.rptr, A.n, False)
    r = ref.amc_permutation(A.cind, A.rptr, A.n, False)
    assert a[0] == r[0] and all(np.array_equal(x, y) for x, y in zip(a[1:], r[1:]))
    nc, sc, LP, RP = a
    Ap, Ar = port.reordering(A, LP, RP), ref.reordering(A, LP, RP)
    assert np.array_equal(Ap.val, Ar.val) and np.array_equal(Ap.cind, Ar.cind)
    for p in (1, 2):
        x, y = port.ilup(A, p), ref.ilup(A, p)
        assert np.array_equal(x.rptr, y.rptr) and np.array_equal(x.cind, y.cind) and np.array_equal(x.val, y.val)
        x, y = port.alloc_level_zero(A, p), ref.alloc_level_zero(A, p)
        assert np.array_equal(x.rptr, y.rptr) and np.array_equal(x.cind, y.cind) and np.array_equal(x.val, y.val)
    for bnl, bnw in [(8, 1), (2, 2), (3, 3)]:
        if A.n % bnl:
            continue
        x, y = port.alloc_block_zero(A, bnl, bnw), ref.alloc_block_zero(A, bnl, bnw)
        assert np.array_equal(x.rptr, y.rptr) and np.array_equal(x.cind, y.cind)
        bx, by = port.csr2bcsr(A, bnl, bnw), ref.csr2bcsr(A, bnl, bnw)
        assert all(np.array_equal(u, v) for u, v in zip(bx, by))
    sx, sy = port.csr2sell(A, 32), ref.csr2sell(A, 32)
    assert all(np.array_equal(u, v) for u, v in zip(sx, sy))
    for key in ("LD-U", "L-DU", "L-D-U", "LU-D"):
        px, rx = port.split(A, key, True), ref.split(A, key, True)
        for u, v in zip(px, rx):
            assert (u is None) == (v is None)
            if u is not None:
                assert all(np.array_equal(p, q) for p, q in zip((u.val, u.cind, u.rptr) if hasattr(u, "val") else (u,),
                                                                (v.val, v.cind, v.rptr) if hasattr(v, "val") else (v,)))


def test_small_ilub_sweeps_match_golden(port, small):
    s = small
    bl = (s["Lb_val"], s["Lb_cind"], s["Lb_rptr"])
    bu = (s["Ub_val"], s["Ub_cind"], s["Ub_rptr"])
    sc = s["size_color"]
    assert np.array_equal(port.ilub_apply(bl, bu, s["v"], 8, 1), s["y_ilub_seq"])
    assert np.array_equal(port.ilub_apply(bl, bu, s["v"], 8, 1, sc, len(sc) - 1, 16), s["y_ilub_abmc"])
    # the first row of the reordered system has no lower entries: Csr2Bcsr gave
    # it a value on the diagonal, and the sweep must differ from the CSR one
    assert bl[0][0] != 0.0
    assert not np.array_equal(s["y_ilub_seq"], s["y_ilu_seq"])


@pytest.mark.parametrize("bnl,bnw", [(1, 1), (2, 1), (2, 2), (3, 3), (4, 1), (4, 2), (8, 1), (8, 2)])
def test_live_ilub_sweeps_match_reference(port, ref, bnl, bnw):
    A = P.convdiff3d(12, 0.5)  # N = 1728: a multiple of every block shape
    N = A.n
    v = np.random.default_rng(3).uniform(-1, 1, N)
    L, U, _ = port.split(port.ilu0(port.alloc_block_zero(A, bnl, bnw)), "L-DU", True)
    bl, bu = port.csr2bcsr(L, bnl, bnw), port.csr2bcsr(U, bnl, bnw)
    assert np.array_equal(port.ilub_apply(bl, bu, v, bnl, bnw), ref.ilub_apply(bl, bu, v, bnl, bnw))
    bs = 24  # a multiple of every bnl
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, N, bs, False, "connect")
    Ar = port.reordering(A, LP, RP)
    L, U, _ = port.split(port.ilu0(port.alloc_block_zero(Ar, bnl, bnw)), "L-DU", True)
    bl, bu = port.csr2bcsr(L, bnl, bnw), port.csr2bcsr(U, bnl, bnw)
    assert np.array_equal(port.ilub_apply(bl, bu, v, bnl, bnw, sc, nc, bs),
                          ref.ilub_apply(bl, bu, v, bnl, bnw, sc, nc, bs))


def test_live_solvers_match_reference(port, ref):
    A = _vs_ref_case()
    N = A.n
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, N, 16, False, "connect")
    Ar = port.reordering(A, LP, RP)
    b = Ar.matvec(P.uniform_solution(N, 0)[LP])
    nb = float(np.sqrt(np.dot(b, b)))
    L, U, _ = port.split(port.ilu0(Ar), "L-DU", True)
    xr = np.zeros(N)
    t = ref.solve_text("abmc_ilu_gmres_d", Ar.val, Ar.cind, Ar.rptr, L.val, L.cind, L.rptr, U.val,
                       U.cind, U.rptr, sc, nc, 16, b, xr, nb, 100, 30, N, 1e-8)
    x, it, res, _ = port.solve("gmres", Ar, b, L=L, U=U, pc=oracle.PC_ILU_ABMC, cptr=sc, cnum=nc, bsize=16,
                               outer=100, m=30, eps=1e-8, nrm_b=nb)
    assert it == oracle.parse_solver_stdout(t)["iters"]
    np.testing.assert_allclose(x, xr, rtol=0, atol=1e-11)
    xr = np.zeros(N)
    t = ref.solve_text("ilu_gcr_d", Ar.val, Ar.cind, Ar.rptr, L.val, L.cind, L.rptr, U.val, U.cind, U.rptr,
                       b, xr, nb, 100, 20, N, 1e-8)
    x, it, res, _ = port.solve("gcr", Ar, b, L=L, U=U, pc=oracle.PC_ILU, outer=100, m=20, eps=1e-8, nrm_b=nb)
    assert it == oracle.parse_solver_stdout(t)["iters"]
    np.testing.assert_allclose(x, xr, rtol=0, atol=1e-11)


def test_block27_generator_and_live_ilub33_gcr(port, ref):
    A = P.block27(4, seed=3)
    assert A.n == 192 and np.all(np.diff(A.rptr) % 3 == 0)
    Lf, Uf, _ = port.split(port.ilu0(port.alloc_block_zero(A, 3, 3)), "L-DU", True)
    bl, bu = port.csr2bcsr(Lf, 3, 3), port.csr2bcsr(Uf, 3, 3)
    assert all(np.array_equal(p, q) for p, q in zip(bl, ref.csr2bcsr(Lf, 3, 3)))
    b = A.matvec(np.ones(A.n))
    nb = float(np.linalg.norm(b))
    _, it, _, _ = port.solve("gcr", A, b, L=bl, U=bu, pc=oracle.PC_ILUB, bnl=3, bnw=3, outer=100, m=20, eps=1e-8)
    txt = ref.solve_text("ilub_gcr_d", A.val, A.cind, A.rptr, *bl, *bu, b, np.zeros(A.n), nb, 100, 20, A.n, 1e-8,
                         3, 3)
    assert it == oracle.parse_solver_stdout(txt)["iters"]
