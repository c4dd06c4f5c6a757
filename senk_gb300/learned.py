"""The learned preconditioner from Python: the network object over the C ABI
(senk_mpnn_*), the seeded problem family it is trained on, and the training
and evaluation loops (flexible GCR(m) with K = ILU + net against plain
ILU-GCR(m)).

The network runs on the GPU only: its forward, backward and Adam kernels are in
csrc/mpnn.cu. This module only sequences calls and prepares host inputs.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from . import problems as P
from . import setup as S
from .lib import PC_ILU_ABMC, Result, check, lib
from .solver import System

HID, LAYERS, NIN = 64, 4, 3
OFF_WIN = 0
OFF_BIN = OFF_WIN + NIN * HID
OFF_LAYER = OFF_BIN + HID
LAYER_SIZE = 2 * HID * HID + HID
OFF_WOUT = OFF_LAYER + LAYERS * LAYER_SIZE
OFF_BOUT = OFF_WOUT + HID
NPARAMS = OFF_BOUT + 1


def init_params(seed: int = 0) -> np.ndarray:
    """He-scaled hidden weights, zero output layer: the untrained network adds
    nothing, so K starts as plain ILU(0)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float32)
    p[OFF_WIN:OFF_BIN] = rng.normal(0, np.sqrt(2.0 / NIN), NIN * HID)
    for l in range(LAYERS):
        o = OFF_LAYER + l * LAYER_SIZE
        p[o:o + 2 * HID * HID] = rng.normal(0, 0.5 * np.sqrt(2.0 / (2 * HID)), 2 * HID * HID)
    return p


class Net:
    """A senk_mpnn handle."""

    def __init__(self, params: np.ndarray | None = None, seed: int = 0):
        assert lib().senk_mpnn_num_params() == NPARAMS
        p = init_params(seed) if params is None else np.ascontiguousarray(params, np.float32)
        self._h = C.c_void_p()
        check("senk_mpnn_create", lib().senk_mpnn_create(C.byref(self._h), p.ctypes.data_as(C.c_void_p), NPARAMS))

    @property
    def params(self) -> np.ndarray:
        p = np.empty(NPARAMS, np.float32)
        check("senk_mpnn_get_params", lib().senk_mpnn_get_params(self._h, p.ctypes.data_as(C.c_void_p), NPARAMS))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check("senk_mpnn_set_params", lib().senk_mpnn_set_params(self._h, p.ctypes.data_as(C.c_void_p), NPARAMS))

    def set_loss(self, mode: int):
        """Training objective: 1 = residual space (default), 0 = error space."""
        check("senk_mpnn_set_loss", lib().senk_mpnn_set_loss(self._h, mode))

    def set_step(self, mode: int):
        """Step of the correction in the GCR: 0 = ILU + c, 1 = ILU + alpha c with
        the least-squares alpha."""
        check("senk_mpnn_set_step", lib().senk_mpnn_set_step(self._h, mode))

    def bind(self, sysm: System):
        check("senk_mpnn_bind", lib().senk_mpnn_bind(self._h, sysm._h))

    def loss_grad(self, sysm: System, r_dev: int, e_dev: int, want_grad=True):
        loss = C.c_double()
        g = np.empty(NPARAMS, np.float32) if want_grad else None
        check("senk_mpnn_loss_grad", lib().senk_mpnn_loss_grad(
            self._h, sysm._h, r_dev, e_dev, C.byref(loss), None if g is None else g.ctypes.data_as(C.c_void_p)))
        return loss.value, g

    def train_step(self, sysm: System, r_dev: int, e_dev: int, lr: float) -> float:
        loss = C.c_double()
        check("senk_mpnn_train_step", lib().senk_mpnn_train_step(self._h, sysm._h, r_dev, e_dev, lr,
                                                                 C.byref(loss)))
        return loss.value

    def apply(self, sysm: System, r_dev: int, out_dev: int):
        check("senk_mpnn_apply", lib().senk_mpnn_apply(self._h, sysm._h, r_dev, out_dev))

    def attach(self, sysm: System, stall: float = 0.9):
        check("senk_system_set_learned", lib().senk_system_set_learned(sysm._h, self._h, stall))

    @staticmethod
    def detach(sysm: System):
        check("senk_system_set_learned", lib().senk_system_set_learned(sysm._h, None, 0.9))

    def close(self):
        if self._h:
            lib().senk_mpnn_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ problem family

@dataclass
class Member:
    """One system of the family: ABMC-ordered A, its ILU(0) factors, b, x_true."""
    seed: int
    sigma: float
    corr: float
    A: P.Csr
    L: P.Csr
    U: P.Csr
    cptr: np.ndarray
    cnum: int
    b: np.ndarray
    x_true: np.ndarray


def family_member(n: int, seed: int, bsize: int = 16) -> Member:
    """3D 7-point diffusion on n^3 with coefficients exp(g): g a Gaussian random
    field with sigma ~ U[0.5, 2.0] and correlation length ~ U[4, 16] cells drawn
    from the seed; x_true ~ N(0, 1); ABMC (bsize 16) ordering and ILU(0)."""
    rng = np.random.default_rng([seed, 0x5E11])
    sigma = float(rng.uniform(0.5, 2.0))
    corr = float(rng.uniform(4.0, 16.0))
    A = P.vardiff3d(n, sigma, corr, seed)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, bsize, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    L, U, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    xt = P.normal_solution(A.n, seed)[LP]
    return Member(seed, sigma, corr, Ar, L, U, sc, nc, Ar.matvec(xt), xt)


def make_system(mb: Member, m_max: int = 0) -> System:
    return System(mb.A, mb.L, mb.U, PC_ILU_ABMC, mb.cptr, mb.cnum, 16, m_max=m_max)


# ------------------------------------------------------------------ training

def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def residual_error_pairs(torch, mb: Member, sysm: System, cycles=(1, 2, 3, 4), m: int = 10):
    """(r_k, e_k) device pairs from plain ILU(0)-GMRES(m) iterates x_k taken
    after the given numbers of restart cycles (x_0 = 0). The default leaves out
    x_0: its residual b = A x_true (x_true white noise) is far rougher than any
    the preconditioner meets once the iteration runs, and fitting it costs the
    fit on all the others."""
    b = _dev(torch, mb.b)
    xt = _dev(torch, mb.x_true)
    A = mb.A
    val, cind, rptr = _dev(torch, A.val), torch.from_numpy(A.cind).cuda(), torch.from_numpy(A.rptr).cuda()
    sysm.set_rhs(mb.b)
    nb = float(np.linalg.norm(mb.b))
    done = 0
    out = []
    for k in sorted(cycles):
        if k > done:
            sysm.gmres(nb, k - done, m, 1e-14)
            done = k
        x = sysm.get_x()
        xd = _dev(torch, x)
        ax = torch.zeros_like(xd)
        check("spmv", lib().senk_dev_spmv_csr_d(val.data_ptr(), cind.data_ptr(), rptr.data_ptr(), xd.data_ptr(),
                                                ax.data_ptr(), A.n, A.nnz, None))
        torch.cuda.synchronize()
        out.append((b - ax, xt - xd))
    return out


def train(torch, net: Net, n: int, seeds, epochs: int = 1, lr: float = 3e-4, cycles=(1, 2, 3, 4),
          log=None) -> list:
    """Online training: for each system of the family, generate its pairs on the
    GPU and take one Adam step per pair (pairs are not kept)."""
    losses = []
    for ep in range(epochs):
        for s in seeds:
            mb = family_member(n, s)
            sysm = make_system(mb, m_max=10)
            net.bind(sysm)
            for r, e in residual_error_pairs(torch, mb, sysm, cycles):
                losses.append(net.train_step(sysm, r.data_ptr(), e.data_ptr(), lr))
            sysm.close()
            if log:
                log(f"epoch {ep} seed {s}: loss {np.mean(losses[-len(cycles):]):.4f}")
    return losses


def compare_gcr(net: Net, mb: Member, m: int = 20, eps: float = 1e-8, max_outer: int = 500, stall: float = 0.9,
                fixed_cycles: int = 0, gmres_m: int = 0):
    """Plain ILU(0)-GCR(m) and flexible GCR(m) with K = ILU + net on one system:
    iterations, solve ms, FP64 true residuals, and the fall-back cycle. With
    fixed_cycles, both also run exactly that many restart cycles and report the
    FP64 true residual reached (finer than GCR's restart-granular counts); with
    gmres_m, plain FP64 ILU(0)-GMRES(gmres_m) on the same system is timed too."""
    sysm = make_system(mb, m_max=gmres_m)
    nb = float(np.linalg.norm(mb.b))

    def true_res(x):
        return float(np.linalg.norm(mb.b - mb.A.matvec(x)) / nb)

    def after_cycles():
        sysm.set_rhs(mb.b)
        sysm.gcr(nb, fixed_cycles, m, 1e-300)
        return true_res(sysm.get_x())

    out = {}
    if gmres_m:
        sysm.set_rhs(mb.b)
        sysm.gmres(nb, 10000 // gmres_m, gmres_m, eps)  # warm-up
        sysm.set_rhs(mb.b)
        rg: Result = sysm.gmres(nb, 10000 // gmres_m, gmres_m, eps)
        out["gmres"] = dict(iters=rg.iters, ms=rg.solve_ms, converged=bool(rg.converged),
                            true_res=true_res(sysm.get_x()))
    sysm.set_rhs(mb.b)
    sysm.gcr(nb, max_outer, m, eps)  # warm-up (graph capture)
    sysm.set_rhs(mb.b)
    r0: Result = sysm.gcr(nb, max_outer, m, eps)
    out["plain"] = dict(iters=r0.iters, ms=r0.solve_ms, converged=bool(r0.converged), true_res=true_res(sysm.get_x()))
    if fixed_cycles:
        out["plain"]["res_after_cycles"] = after_cycles()
    net.bind(sysm)
    net.attach(sysm, stall)
    sysm.set_rhs(mb.b)
    sysm.gcr(nb, max_outer, m, eps)
    sysm.set_rhs(mb.b)
    t0 = time.perf_counter()
    r1: Result = sysm.gcr(nb, max_outer, m, eps)
    out["learned"] = dict(iters=r1.iters, ms=r1.solve_ms, converged=bool(r1.converged),
                          true_res=true_res(sysm.get_x()), wall_ms=1e3 * (time.perf_counter() - t0),
                          fallback_cycle=lib().senk_system_learned_fallback(sysm._h))
    if fixed_cycles:
        net.attach(sysm, 1.0)  # fall back only on a cycle without any progress
        out["learned"]["res_after_cycles"] = after_cycles()
    Net.detach(sysm)
    sysm.close()
    return out


def bytes_per_application(n: int, nnz: int) -> dict:
    """Bytes one application of the network moves (at least once each), against
    one FP64 ILU(0) application and one FP64 SpMV on the same graph (n nodes,
    nnz entries of A): FP32 activations H (64 per node), BF16 GEMM operands X
    (128 per node: h and the aggregate m), the row-normalised graph (value and
    column per entry), per layer the aggregate's gathers of neighbours' h rows,
    its m output, and the GEMM's X read, H read, H and next X written."""
    layers, hid = LAYERS, HID
    graph = nnz * 8 + (n + 1) * 4
    streamed = graph + n * hid * 2 + n * 2 * hid * 2 + n * hid * 4 * 2 + n * hid * 2  # per layer, HBM
    gathers = nnz * hid * 2                                                          # per layer, mostly L2
    encode = n * (8 + 8) + n * hid * (4 + 2)
    decode = n * hid * 4 + n * 8 * 2
    net = encode + layers * streamed + decode
    ilu = nnz * 12 + n * 8 * 5
    spmv = nnz * 12 + 4 * (n + 1) + 16 * n
    return {"network_streamed": int(net), "network_gathers": int(layers * gathers), "ilu0_fp64": int(ilu),
            "spmv_fp64": int(spmv), "network_over_ilu": round(net / ilu, 1)}


def main(argv=None):
    """Train on the seeded family and compare flexible GCR(m) with K = ILU + net
    against plain ILU(0)-GCR(m) on held-out seeds; prints one JSON line.

        python -m senk_gb300.learned --n 32 --train 64 --epochs 2 --test 4
    """
    import argparse
    import json

    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=32, help="grid points per dimension")
    ap.add_argument("--train", type=int, default=64, help="training systems (seeds 1000..)")
    ap.add_argument("--epochs", type=int, default=2)
    ap.add_argument("--test", type=int, default=4, help="held-out systems (seeds 900000..)")
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--clip", type=float, default=1.0)
    ap.add_argument("--m", type=int, default=20)
    ap.add_argument("--loss", type=int, default=1, help="1 residual space, 0 error space")
    ap.add_argument("--save", default=None, help="write the trained parameters (.npy)")
    ap.add_argument("--step", type=int, default=1, help="0: fixed step, 1: least-squares step of the correction")
    ap.add_argument("--fixed-cycles", type=int, default=3, help="also compare residuals after this many cycles")
    ap.add_argument("--gmres", type=int, default=30, help="also time plain FP64 ILU(0)-GMRES(m) (0: no)")
    ap.add_argument("--load", default=None, help="start from these parameters (.npy)")
    args = ap.parse_args(argv)
    net = Net(np.load(args.load) if args.load else None, seed=0)
    net.set_loss(args.loss)
    net.set_step(args.step)
    check("senk_mpnn_set_clip", lib().senk_mpnn_set_clip(net._h, args.clip))
    t0 = time.perf_counter()
    losses = train(torch, net, args.n, range(1000, 1000 + args.train), args.epochs, args.lr) if args.train else [0.0]
    train_s = time.perf_counter() - t0
    results = []
    for s in range(900000, 900000 + args.test):
        results.append(dict(seed=s, **compare_gcr(net, family_member(args.n, s), m=args.m,
                                                  fixed_cycles=args.fixed_cycles, gmres_m=args.gmres)))
    if args.save:
        np.save(args.save, net.params)
    plain = [r["plain"]["iters"] for r in results]
    learned = [r["learned"]["iters"] for r in results]
    out = dict(n=args.n, train_systems=args.train, epochs=args.epochs, pairs=len(losses), train_s=round(train_s, 1),
               loss_first=float(np.mean(losses[:8])), loss_last=float(np.mean(losses[-8:])),
               plain_iters=plain, learned_iters=learned,
               plain_ms=[round(r["plain"]["ms"], 2) for r in results],
               learned_ms=[round(r["learned"]["ms"], 2) for r in results],
               learned_true_res=[r["learned"]["true_res"] for r in results],
               fallback=[r["learned"]["fallback_cycle"] for r in results])
    if args.fixed_cycles:
        out["plain_res_after_cycles"] = [r["plain"]["res_after_cycles"] for r in results]
        out["learned_res_after_cycles"] = [r["learned"]["res_after_cycles"] for r in results]
    if args.gmres:
        out["gmres_fp64_iters"] = [r["gmres"]["iters"] for r in results]
        out["gmres_fp64_ms"] = [round(r["gmres"]["ms"], 2) for r in results]
    mb = family_member(args.n, 900000) if args.test else None
    if mb is not None:
        out["bytes_per_application"] = bytes_per_application(mb.A.n, mb.A.nnz)
    print(json.dumps(out))
    net.close()


if __name__ == "__main__":
    main()
