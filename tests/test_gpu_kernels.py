"""GPU kernels through the C ABI against the oracle (FP64 within 1e-12 relative,
FP32 within 1e-5 relative, in the infinity norm)."""
import ctypes as C

import numpy as np
import pytest

from senk_gb300 import lib as L
from senk_gb300 import problems as P
from senk_gb300 import setup as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


def rel(a, b):
    d = np.max(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)))
    s = np.max(np.abs(np.asarray(b, np.float64)))
    return d / (s if s > 0 else 1.0)


CASES = {
    "poisson128": lambda: P.poisson2d(128),
    "poisson10": lambda: P.poisson2d(10),
    "convdiff24": lambda: P.convdiff3d(24, 0.5),
    "vardiff16": lambda: P.vardiff3d(16, 1.5, 4.0, 3),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_spmv_csr_f64(torch, port, case):
    A = CASES[case]()
    x = np.random.default_rng(1).uniform(-1, 1, A.n)
    v, c, r, xd = dev(torch, A.val), dev(torch, A.cind), dev(torch, A.rptr), dev(torch, x)
    y = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("spmv", L.lib().senk_dev_spmv_csr_d(v.data_ptr(), c.data_ptr(), r.data_ptr(), xd.data_ptr(),
                                                 y.data_ptr(), A.n, A.nnz, None))
    torch.cuda.synchronize()
    assert rel(host(y), port.spmv_csr(A, x)) <= 1e-12


@pytest.mark.parametrize("case", ["poisson128", "convdiff24"])
def test_spmv_csr_f32(torch, port, case):
    A = CASES[case]().astype(np.float32)
    x = np.random.default_rng(2).uniform(-1, 1, A.n).astype(np.float32)
    v, c, r, xd = dev(torch, A.val), dev(torch, A.cind), dev(torch, A.rptr), dev(torch, x)
    y = torch.zeros(A.n, dtype=torch.float32, device="cuda")
    L.check("spmv", L.lib().senk_dev_spmv_csr_s(v.data_ptr(), c.data_ptr(), r.data_ptr(), xd.data_ptr(),
                                                 y.data_ptr(), A.n, A.nnz, None))
    torch.cuda.synchronize()
    assert rel(host(y), port.spmv_csr(A, x)) <= 1e-5


def test_spmv_golden(torch, small):
    A = P.Csr(small["Ar_val"], small["Ar_cind"], small["Ar_rptr"])
    v, c, r, xd = dev(torch, A.val), dev(torch, A.cind), dev(torch, A.rptr), dev(torch, small["v"])
    y = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("spmv", L.lib().senk_dev_spmv_csr_d(v.data_ptr(), c.data_ptr(), r.data_ptr(), xd.data_ptr(),
                                                 y.data_ptr(), A.n, A.nnz, None))
    torch.cuda.synchronize()
    assert rel(host(y), small["y_spmv"]) <= 1e-12


def test_spmv_sell_reference_layout(torch, port):
    A = P.convdiff3d(16, 0.5)  # N = 4096, a multiple of the slice length
    sv, sc, sl = port.csr2sell(A, 32)
    x = np.random.default_rng(3).uniform(-1, 1, A.n)
    t = [dev(torch, a) for a in (sv, sc, sl, x)]
    y = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("sell", L.lib().senk_dev_spmv_sell_d(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 32,
                                                  t[3].data_ptr(), y.data_ptr(), A.n, None))
    torch.cuda.synchronize()
    assert rel(host(y), port.spmv_csr(A, x)) <= 1e-12


@pytest.mark.parametrize("bnl,bnw", [(3, 3), (8, 1), (2, 2), (4, 1)])
def test_spmv_bcsr(torch, port, bnl, bnw):
    A = P.convdiff3d(12, 0.5)  # N = 1728
    bv, bc, br = S.Csr2Bcsr(A, bnl, bnw)
    x = np.random.default_rng(4).uniform(-1, 1, A.n)
    t = [dev(torch, a) for a in (bv, bc, br, x)]
    y = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("bcsr", L.lib().senk_dev_spmv_bcsr_d(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(),
                                                  t[3].data_ptr(), y.data_ptr(), A.n, bnl, bnw, None))
    torch.cuda.synchronize()
    assert rel(host(y), port.spmv_bcsr(bv, bc, br, x, A.n, bnl, bnw)) <= 1e-12


def test_bcsr_unsupported_shape_is_rejected(torch):
    z = torch.zeros(10, dtype=torch.float64, device="cuda")
    code = L.lib().senk_dev_spmv_bcsr_d(z.data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(),
                                        10, 5, 2, None)
    assert code == L.ERR_ARG


@pytest.mark.parametrize("n", [1, 31, 1000, 2_000_003])
def test_blas1(torch, n):
    rng = np.random.default_rng(n)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    xd, yd = dev(torch, x), dev(torch, y)
    out = C.c_double()
    L.check("dot", L.lib().senk_dev_dot_d(xd.data_ptr(), yd.data_ptr(), n, C.byref(out), None))
    assert abs(out.value - np.dot(x, y)) <= 1e-12 * max(1.0, np.abs(x * y).sum())
    L.check("nrm2", L.lib().senk_dev_nrm2_d(xd.data_ptr(), n, C.byref(out), None))
    assert abs(out.value - np.linalg.norm(x)) <= 1e-13 * np.linalg.norm(x)
    z = torch.zeros(n, dtype=torch.float64, device="cuda")
    L.check("axpyz", L.lib().senk_dev_axpyz_d(0.5, xd.data_ptr(), yd.data_ptr(), z.data_ptr(), n, None))
    L.check("axpy", L.lib().senk_dev_axpy_d(-2.0, xd.data_ptr(), yd.data_ptr(), n, None))
    torch.cuda.synchronize()
    assert rel(host(z), 0.5 * x + y) <= 1e-15
    assert rel(host(yd), y - 2.0 * x) <= 1e-15
    L.check("axpby", L.lib().senk_dev_axpby_d(3.0, xd.data_ptr(), -1.0, yd.data_ptr(), n, None))
    L.check("scal", L.lib().senk_dev_scal_d(0.25, yd.data_ptr(), n, None))
    L.check("copy", L.lib().senk_dev_copy_d(yd.data_ptr(), z.data_ptr(), n, None))
    torch.cuda.synchronize()
    want = 0.25 * (3.0 * x - (y - 2.0 * x))
    assert rel(host(z), want) <= 1e-15


def _factors(A, sched, bsize=16):
    """(reordered A, L, U, cptr, cnum, precond kind) for a schedule."""
    if sched == "natural":
        L_, U_, _ = S.Split(S.Ilu0(A), "L-DU", True)
        return A, L_, U_, None, 0, L.PC_ILU, 1
    if sched == "amc":
        nc, sc, LP, RP = S.GetAMCPermutation(A.cind, A.rptr, A.n, False)
        kind, bs = L.PC_ILU_AMC, 1
    else:
        nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bsize, False, "connect")
        kind, bs = L.PC_ILU_ABMC, bsize
    Ar = S.Reordering(A, LP, RP)
    L_, U_, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    return Ar, L_, U_, sc, nc, kind, bs


class Plan:
    def __init__(self, L_, U_, kind, sc, nc, bs, dtype=np.float64, sweep=L.SWEEP_AUTO):
        self.h = C.c_void_p()
        T = dtype
        self.keep = [np.ascontiguousarray(a) for a in (L_.val.astype(T), L_.cind, L_.rptr, U_.val.astype(T),
                                                       U_.cind, U_.rptr)]
        cp = None if sc is None else np.ascontiguousarray(sc, np.int32)
        self.keep.append(cp)
        self.code = L.lib().senk_ilu_plan_create_sched(C.byref(self.h), L.F32 if T == np.float32 else L.F64, L_.n,
                                                       *[L.ptr(a) for a in self.keep[:6]], kind, L.ptr(cp), nc, bs,
                                                       sweep)

    def __del__(self):
        if self.h:
            L.lib().senk_ilu_plan_destroy(self.h)


def _ragged(n=3001, seed=11):
    """A nonsymmetric matrix whose rows hold 1 to 40 entries (diagonal first),
    N not a multiple of 32: sigma sorting permutes its rows."""
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for i in range(n):
        k = int(rng.integers(0, 40))
        c = np.unique(np.concatenate([[i], rng.integers(0, n, k)]))
        rows.append(len(c))
        cols.append(c)
        vals.append(np.where(c == i, 50.0, rng.uniform(-1, 1, len(c))))
    rptr = np.concatenate([[0], np.cumsum(rows)]).astype(np.int32)
    return P.Csr(np.concatenate(vals), np.concatenate(cols).astype(np.int32), rptr)


@pytest.mark.parametrize("fmt", [L.SPMV_AUTO, L.SPMV_SELL_SIGMA, L.SPMV_SELL, L.SPMV_CSR])
@pytest.mark.parametrize("case", ["ragged", "convdiff24", "poisson10"])
def test_system_spmv_formats(torch, port, case, fmt):
    """The solver's own SpMV (senk_system_apply_a) in each format, SELL-32-sigma
    (the default) included, against the oracle's CSR SpMV; and, on the ragged
    and small Poisson matrices, a GMRES(30) solve with that format within 2
    iterations of the oracle's count (the residual kernel takes the same row
    map)."""
    from senk_gb300.solver import System
    A = _ragged() if case == "ragged" else CASES[case]()
    x = np.random.default_rng(4).uniform(-1, 1, A.n)
    want = port.spmv_csr(A, x)
    for T, tol in ((np.float64, 1e-12), (np.float32, 1e-5)):
        sy = System(A, dtype=T, m_max=30, spmv=fmt)
        got = sy.apply_a(x.astype(T))
        sy.close()
        assert rel(got, want) <= tol, (T, rel(got, want))
    if case == "convdiff24":
        return  # unpreconditioned GMRES runs long there; the solve check uses the other two
    b = port.spmv_csr(A, np.ones(A.n))
    nb = float(np.linalg.norm(b))
    sy = System(A, dtype=np.float64, m_max=30, spmv=fmt)
    sy.set_rhs(b)
    r = sy.gmres(nb, 40, 30, 1e-8)
    sy.close()
    _, it, _, _ = port.solve("gmres", A, b, outer=40, m=30, eps=1e-8, nrm_b=nb)
    assert r.converged and abs(r.iters - it) <= 2, (r.iters, it)


SWEEPS = [("natural", 16), ("amc", 16), ("abmc", 16), ("abmc", 8), ("abmc", 32), ("abmc", 4), ("abmc", 2)]


@pytest.mark.parametrize("sweep", [L.SWEEP_AUTO, L.SWEEP_DATAFLOW, L.SWEEP_COLOURS, L.SWEEP_COMPACT,
                                   L.SWEEP_PERSISTENT, L.SWEEP_WIDE, L.SWEEP_ROWS, L.SWEEP_ROWS_WIDE])
@pytest.mark.parametrize("case", ["poisson128", "convdiff24", "vardiff16"])
@pytest.mark.parametrize("sched,bsize", SWEEPS)
def test_ilu_sweeps_f64(torch, port, case, sched, bsize, sweep):
    A = CASES[case]()
    if sched == "abmc" and A.n % bsize:
        pytest.skip("N not a multiple of bsize")
    if sched == "natural" and sweep == L.SWEEP_COLOURS:
        pytest.skip("the natural order has one schedule (level sets)")
    Ar, L_, U_, sc, nc, kind, bs = _factors(A, sched, bsize)
    pl = Plan(L_, U_, kind, sc, nc, bs, sweep=sweep)
    L.check("plan", pl.code)
    v = np.random.default_rng(5).uniform(-1, 1, A.n)
    xd = dev(torch, v)
    yd = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
    tl = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("sweepL", L.lib().senk_ilu_plan_sweep(pl.h, 0, xd.data_ptr(), tl.data_ptr(), None))
    torch.cuda.synchronize()
    want_l = port.sptrsv(L_, v, False)
    want = port.sptrsv(U_, want_l, True)
    assert rel(host(tl), want_l) <= 1e-12
    assert rel(host(yd), want) <= 1e-12
    # in place: x == y, twice (the dataflow sweeps start a new epoch each time)
    x2 = xd.clone()
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), xd.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel(host(xd), want) <= 1e-12
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, x2.data_ptr(), x2.data_ptr(), None))
    L.check("status", L.lib().senk_ilu_plan_status(pl.h, None))
    assert rel(host(x2), want) <= 1e-12


@pytest.mark.parametrize("sweep", [L.SWEEP_AUTO, L.SWEEP_DATAFLOW, L.SWEEP_COLOURS, L.SWEEP_COMPACT,
                                   L.SWEEP_PERSISTENT, L.SWEEP_WIDE, L.SWEEP_ROWS, L.SWEEP_ROWS_WIDE])
@pytest.mark.parametrize("sched,bsize", [("abmc", 16), ("natural", 16), ("amc", 16), ("abmc", 4)])
def test_ilu_sweeps_f32(torch, port, sched, bsize, sweep):
    A = P.convdiff3d(24, 0.5)
    Ar, L_, U_, sc, nc, kind, bs = _factors(A, sched, bsize)
    pl = Plan(L_, U_, kind, sc, nc, bs, np.float32, sweep=sweep)
    L.check("plan", pl.code)
    v = np.random.default_rng(6).uniform(-1, 1, A.n).astype(np.float32)
    xd = dev(torch, v)
    yd = torch.zeros(A.n, dtype=torch.float32, device="cuda")
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
    torch.cuda.synchronize()
    want = port.ilu_apply(L_.astype(np.float32), U_.astype(np.float32), v, dtype=np.float32)
    assert rel(host(yd), want) <= 1e-5


def test_ilu_sweep_golden(torch, small):
    s = small
    L_ = P.Csr(s["L_val"], s["L_cind"], s["L_rptr"])
    U_ = P.Csr(s["U_val"], s["U_cind"], s["U_rptr"])
    sc = s["size_color"]
    pl = Plan(L_, U_, L.PC_ILU_ABMC, sc, len(sc) - 1, 16)
    L.check("plan", pl.code)
    xd = dev(torch, s["v"])
    yd = torch.zeros(L_.n, dtype=torch.float64, device="cuda")
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel(host(yd), s["y_ilu_abmc"]) <= 1e-12
    assert rel(host(yd), s["y_ilu_seq"]) <= 1e-12


def test_ilu_sweep_at_benchmark_size(torch, port):
    """The 64^3 convection-diffusion system (16,384 chains, 11 colours) against
    the oracle under the default, dataflow, compact, cooperative,
    two-rows-per-thread and row-per-lane schedules, FP64 and FP32, several
    applications in a row."""
    A = P.convdiff3d(64, 0.5)
    Ar, L_, U_, sc, nc, kind, bs = _factors(A, "abmc", 16)
    v = np.random.default_rng(9).uniform(-1, 1, A.n)
    want = port.sptrsv(U_, port.sptrsv(L_, v, False), True)
    for T, tol, sweep in ((np.float64, 1e-12, L.SWEEP_AUTO), (np.float32, 1e-5, L.SWEEP_AUTO),
                          (np.float64, 1e-12, L.SWEEP_DATAFLOW), (np.float32, 1e-5, L.SWEEP_COMPACT),
                          (np.float64, 1e-12, L.SWEEP_PERSISTENT), (np.float32, 1e-5, L.SWEEP_PERSISTENT),
                          (np.float64, 1e-12, L.SWEEP_WIDE), (np.float32, 1e-5, L.SWEEP_WIDE),
                          (np.float64, 1e-12, L.SWEEP_ROWS), (np.float32, 1e-5, L.SWEEP_ROWS),
                          (np.float32, 1e-5, L.SWEEP_ROWS_WIDE)):
        pl = Plan(L_, U_, kind, sc, nc, bs, T, sweep=sweep)
        L.check("plan", pl.code)
        xd = dev(torch, v.astype(T))
        yd = torch.zeros(A.n, dtype=xd.dtype, device="cuda")
        for _ in range(3):
            L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
        L.check("status", L.lib().senk_ilu_plan_status(pl.h, None))
        if T == np.float32:
            want32 = port.ilu_apply(L_.astype(np.float32), U_.astype(np.float32), v.astype(np.float32),
                                    dtype=np.float32)
            assert rel(host(yd), want32) <= tol
        else:
            assert rel(host(yd), want) <= tol


def test_dataflow_wait_that_runs_out_is_reported(torch):
    """A group made to wait on its own flag (which nothing sets in time) gives up
    after its bounded wait; the call reports the failure, the device stays usable,
    and a fresh plan sweeps correctly afterwards."""
    A = P.convdiff3d(24, 0.5)
    Ar, L_, U_, sc, nc, kind, bs = _factors(A, "abmc", 16)
    pl = Plan(L_, U_, kind, sc, nc, bs, sweep=L.SWEEP_DATAFLOW)
    L.check("plan", pl.code)
    # a group of a later colour (one that reads other groups)
    assert any(L.lib().senk_ilu_plan_test_stall(pl.h, 0, g) == L.OK for g in range(12, 0, -1))
    v = np.random.default_rng(8).uniform(-1, 1, A.n)
    xd = dev(torch, v)
    yd = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
    code = L.lib().senk_ilu_plan_status(pl.h, None)
    assert code == L.ERR_CUDA
    assert "wait" in L.lib().senk_last_error().decode()
    torch.cuda.synchronize()
    pl2 = Plan(L_, U_, kind, sc, nc, bs, sweep=L.SWEEP_DATAFLOW)
    L.check("plan", pl2.code)
    L.check("apply", L.lib().senk_ilu_plan_apply(pl2.h, xd.data_ptr(), yd.data_ptr(), None))
    L.check("status", L.lib().senk_ilu_plan_status(pl2.h, None))


def test_cooperative_barrier_wait_that_runs_out_is_reported(torch, port):
    """The cooperative sweep's first grid barrier made to wait for more arrivals
    than there are CTAs: every CTA gives up after its bounded wait, the call
    reports the failure, the device stays usable, and the plan's next sweep (the
    launch that gave up reset the barrier words) is correct."""
    A = P.convdiff3d(24, 0.5)
    Ar, L_, U_, sc, nc, kind, bs = _factors(A, "abmc", 16)
    pl = Plan(L_, U_, kind, sc, nc, bs, sweep=L.SWEEP_PERSISTENT)
    L.check("plan", pl.code)
    L.check("stall", L.lib().senk_ilu_plan_test_stall(pl.h, 1, 0))
    v = np.random.default_rng(8).uniform(-1, 1, A.n)
    xd = dev(torch, v)
    yd = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
    assert L.lib().senk_ilu_plan_status(pl.h, None) == L.ERR_CUDA
    assert "wait" in L.lib().senk_last_error().decode()
    L.check("apply", L.lib().senk_ilu_plan_apply(pl.h, xd.data_ptr(), yd.data_ptr(), None))
    L.check("status", L.lib().senk_ilu_plan_status(pl.h, None))
    torch.cuda.synchronize()
    assert rel(host(yd), port.sptrsv(U_, port.sptrsv(L_, v, False), True)) <= 1e-12


def test_plan_rejects_bad_schedules():
    A = P.convdiff3d(12, 0.5)
    Ar, L_, U_, sc, nc, kind, bs = _factors(A, "abmc", 16)
    assert Plan(L_, U_, kind, sc, nc, 12).code == L.ERR_ARG       # chain length not a power of two
    bad = sc.copy()
    bad[-1] += 1
    assert Plan(L_, U_, kind, bad, nc, 16).code == L.ERR_ARG      # colours do not cover N
    # colouring that does not fit the factor (natural factors, ABMC colours)
    Ln, Un, _ = S.Split(S.Ilu0(A), "L-DU", True)
    assert Plan(Ln, Un, kind, sc, nc, 16).code == L.ERR_ARG
