"""Device diagonal scaling (senk_dev_get_diag / senk_dev_scaling /
senk_dev_diag_scaling, FP64 and FP32) against the host GetDiag / Scaling
(include/senk_matrix.hpp:391-416, pinned to the reference): values bit for
bit. Then the driver's pipeline (main.cpp:11-73) from a MatrixMarket file:
read, ABMC, reorder, scale on the device, ILU(0), GMRES on the GPU, against the
oracle's solve of the same scaled system."""
import numpy as np
import pytest

import oracle
from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S
from senk_gb300 import solver as SV

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes()


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("case", ["vardiff12", "convdiff16", "block27_6"])
def test_device_scaling_is_bit_identical(torch, port, dtype, case):
    A = {"vardiff12": lambda: P.vardiff3d(12, 1.5, 4.0, 3), "convdiff16": lambda: P.convdiff3d(16, 0.5),
         "block27_6": lambda: P.block27(6, seed=1)}[case]()
    sfx = "s" if dtype == np.float32 else "d"
    val = A.val.astype(dtype)
    v, c, r = _dev(torch, val), _dev(torch, A.cind), _dev(torch, A.rptr)
    d = torch.zeros(A.n, dtype=v.dtype, device="cuda")
    L.check("get_diag", getattr(L.lib(), f"senk_dev_get_diag_{sfx}")(v.data_ptr(), c.data_ptr(), r.data_ptr(),
                                                                      d.data_ptr(), A.n, None))
    torch.cuda.synchronize()
    want_d = port.get_diag(A).astype(dtype)
    assert _same(d.cpu().numpy(), want_d)
    rng = np.random.default_rng(4)
    ld = rng.uniform(0.5, 2.0, A.n).astype(dtype)
    rd = rng.uniform(0.5, 2.0, A.n).astype(dtype)
    ldd, rdd = _dev(torch, ld), _dev(torch, rd)  # held until the call has run
    L.check("scaling", getattr(L.lib(), f"senk_dev_scaling_{sfx}")(v.data_ptr(), c.data_ptr(), r.data_ptr(),
                                                                    ldd.data_ptr(), rdd.data_ptr(), A.n, None))
    torch.cuda.synchronize()
    if dtype == np.float64:
        want = port.scaling(A, ld, rd).val
    else:  # (ld_i * a_ij) * rd_j in float32, one rounding per product
        rows = np.repeat(np.arange(A.n), np.diff(A.rptr))
        want = (ld[rows] * val) * rd[A.cind]
    assert _same(v.cpu().numpy(), want)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_device_diag_scaling_matches_the_driver(torch, port, dtype):
    A = P.vardiff3d(10, 1.5, 4.0, 5)
    sfx = "s" if dtype == np.float32 else "d"
    v, c, r = _dev(torch, A.val.astype(dtype)), _dev(torch, A.cind), _dev(torch, A.rptr)
    d = torch.zeros(A.n, dtype=v.dtype, device="cuda")
    L.check("diag_scaling", getattr(L.lib(), f"senk_dev_diag_scaling_{sfx}")(v.data_ptr(), c.data_ptr(),
                                                                              r.data_ptr(), d.data_ptr(), A.n, None))
    torch.cuda.synchronize()
    diag = port.get_diag(A).astype(dtype)
    inv = (dtype(1) / np.sqrt(np.abs(diag))).astype(dtype)
    assert _same(d.cpu().numpy(), inv)
    if dtype == np.float64:
        assert _same(v.cpu().numpy(), port.scaling(A, inv, inv).val)


def test_matrix_market_pipeline_solves_like_the_oracle(torch, port, tmp_path):
    """main.cpp's setup from a file (general storage), with the scaling on the
    device, then ABMC-ILU(0)-GMRES(30) on the GPU against the oracle's solve of
    the host-scaled system."""
    A0 = P.vardiff3d(16, 1.5, 4.0, 7)
    path = tmp_path / "vardiff16.mtx"
    rows = np.repeat(np.arange(A0.n), np.diff(A0.rptr))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n% vardiff3d 16^3\n")
        f.write(f"{A0.n} {A0.n} {A0.nnz}\n")
        for i, j, x in zip(rows, A0.cind, A0.val):
            f.write(f"{i + 1} {j + 1} {x:.17g}\n")
    A, M, sym = S.ReadMatrixMarket(path, True)
    assert not sym and M == A0.n and _same(A.val, A0.val)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    v, c, r = _dev(torch, Ar.val), _dev(torch, Ar.cind), _dev(torch, Ar.rptr)
    d = torch.zeros(Ar.n, dtype=torch.float64, device="cuda")
    L.check("diag_scaling", L.lib().senk_dev_diag_scaling_d(v.data_ptr(), c.data_ptr(), r.data_ptr(), d.data_ptr(),
                                                            Ar.n, None))
    torch.cuda.synchronize()
    As = P.Csr(v.cpu().numpy(), Ar.cind.copy(), Ar.rptr.copy())
    diag = port.get_diag(Ar)
    inv = 1.0 / np.sqrt(np.abs(diag))
    assert _same(As.val, port.scaling(Ar, inv, inv).val)
    Lf, Uf, _ = S.Split(S.Ilu0(As), "L-DU", True)
    b = As.matvec(np.ones(As.n))
    nb = float(np.linalg.norm(b))
    x = np.zeros(As.n)
    res = SV.AbmcIluGmresm(As.val, As.cind, As.rptr, Lf.val, Lf.cind, Lf.rptr, Uf.val, Uf.cind, Uf.rptr, sc, nc, 16,
                           b, x, nb, 10000 // 30, 30, As.n, 1e-8)
    assert res.converged
    _, it, _, conv = port.solve("gmres", As, b, L=Lf, U=Uf, pc=oracle.PC_ILU_ABMC, cptr=sc, cnum=nc, bsize=16,
                                m=30, outer=10000 // 30, eps=1e-8, nrm_b=nb)
    assert conv and abs(res.iters - it) <= 2
    assert port.relative_residual(As, b, x) < 1e-8

