#!/usr/bin/env python
"""Benchmark of the preconditioned Krylov path on one GB300.

Workload (the reference's measured configuration that fits one GPU): 3D 7-point
upwind convection-diffusion on a 128^3 grid (N = 2,097,152, nnz = 14,581,760),
unit diffusion, velocity (1,1,1), cell Peclet 0.5; b = A x_true with
x_true ~ U(-1,1) (seed 0); ABMC ordering with block size 16 ("connect",
A + A^T graph); ILU(0); right-preconditioned GMRES(30) in FP64 to a 1e-8
relative residual (x0 = 0).

A step is one complete solve. ``value`` is the mean time of the mixed-precision
solve (GMRES-IR: FP32 ILU factors, sweeps, inner SpMV and Krylov basis inside an
FP64 refinement loop that stops when the FP64 true residual ||b-Ax||/||b|| is
below 1e-8) with A, the factors, b and the workspaces resident in HBM (CUDA
events on the library's stream); the plain FP64 ABMC-ILU(0)-GMRES(30) solve on
the same GPU is reported beside it (``plain_fp64``). ``e2e`` is the mixed solve
through the drop-in C ABI call with host arrays (upload, factor re-layout, solve
and copy-back of x inside the timed region). Inputs are larger than L2 (A, L, U
and the Krylov bases are about 1.2 GB), so no flush is needed between steps.

    python bench.py [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solve ms to 1e-8 FP64 true rel. residual (ABMC-ILU(0) GMRES(30), mixed-precision GMRES-IR)"
TRAFFIC_JSON = os.path.join(ROOT, "profiles", "traffic.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--n", type=int, default=128, help="grid points per dimension")
    ap.add_argument("--m", type=int, default=30)
    ap.add_argument("--eps", type=float, default=1e-8)
    ap.add_argument("--orth", default="cgs", choices=["cgs", "cgs2", "mgs"])
    ap.add_argument("--spmv", default="auto", choices=["auto", "csr", "sell", "sell_sigma"])
    ap.add_argument("--sweep", default="auto",
                    choices=["auto", "colours", "dataflow", "compact", "persistent", "wide", "rows", "rows_wide"],
                    help="schedule of the ABMC triangular sweeps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner comparison")
    ap.add_argument("--no-kernels", action="store_true", help="skip the per-kernel timings (profiling runs)")
    ap.add_argument("--only", default="both", choices=["both", "mixed", "plain"], help="which solves to time")
    ap.add_argument("--inner-tol", type=float, default=1e-4)
    ap.add_argument("--inner-cycles", type=int, default=2)
    ap.add_argument("--legs", default="bicgstab,c1,c3,c4,learned",
                    help="extra legs beside the headline: bicgstab (BiCGStab on the headline system), c1 (2D "
                         "Poisson 128^2), c3 (variable-coefficient 160^3), c4 (block-3x3 96^3), learned")
    ap.add_argument("--c3-n", type=int, default=160)
    ap.add_argument("--c4-n", type=int, default=96)
    ap.add_argument("--leg-steps", type=int, default=2, help="timed solves per extra leg (after one warm-up)")
    return ap.parse_args()


def workload_name(n):
    return f"convdiff3d {n}^3, Pe 0.5, ABMC bsize 16 (connect), ILU(0), GMRES(30), eps 1e-8, x0=0"


def problem(n):
    from senk_gb300 import problems as P
    A = P.convdiff3d(n, 0.5)
    xt = P.uniform_solution(A.n, 0)
    return A, xt


def setup_gpu(A, xt):
    """Product host setup (include/senk_*.hpp through the C ABI)."""
    from senk_gb300 import setup as S
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    Lf, Uf, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    b = Ar.matvec(xt[LP])
    return Ar, Lf, Uf, nc, sc, b


def setup_oracle(port, A, xt):
    nc, sc, LP, RP = port.abmc_permutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = port.reordering(A, LP, RP)
    Lf, Uf, _ = port.split(port.ilu0(Ar), "L-DU", True)
    b = Ar.matvec(xt[LP])
    return Ar, Lf, Uf, nc, sc, b


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.proc = None
        self.lines = []
        self.device = device

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def learned_leg(n=64, test_seeds=(900000, 900001, 900002)):
    """Held-out systems of the 64^3 variable-coefficient family (the learned
    workload): plain ILU(0)-GCR(20) against flexible GCR(20) with K = ILU + net
    (least-squares step), the network trained on the GPU on 1,000 systems of the
    family (senk_gb300/weights), beside the plain FP64 ILU(0)-GMRES(30) of the
    same system; also the FP64 true residual after 3 restart cycles of each GCR
    and the bytes one application of the network moves against ILU(0)."""
    from senk_gb300 import learned as LN
    params = np.load(os.path.join(ROOT, "senk_gb300", "weights", "mpnn_vardiff64_t2000.npy"))
    net = LN.Net(params)
    net.set_step(1)
    rows, mb = [], None
    for s in test_seeds:
        mb = LN.family_member(n, s)
        rows.append(LN.compare_gcr(net, mb, m=20, fixed_cycles=3, gmres_m=30))
    net.close()
    return {"family": f"vardiff3d {n}^3, sigma~U[0.5,2], corr~U[4,16], ABMC 16, ILU(0), GCR(20), 1e-8",
            "trained_on": "2000 systems x 4 pairs, 1 epoch, on the GPU (senk_gb300/weights/README.md)",
            "plain_iters": [r["plain"]["iters"] for r in rows], "learned_iters": [r["learned"]["iters"] for r in rows],
            "plain_ms": [round(r["plain"]["ms"], 2) for r in rows],
            "learned_ms": [round(r["learned"]["ms"], 2) for r in rows],
            "gmres_fp64_iters": [r["gmres"]["iters"] for r in rows],
            "gmres_fp64_ms": [round(r["gmres"]["ms"], 2) for r in rows],
            "plain_res_after_3_cycles": [r["plain"]["res_after_cycles"] for r in rows],
            "learned_res_after_3_cycles": [r["learned"]["res_after_cycles"] for r in rows],
            "learned_true_res": [r["learned"]["true_res"] for r in rows],
            "plain_true_res": [r["plain"]["true_res"] for r in rows],
            "bytes_per_application": LN.bytes_per_application(mb.A.n, mb.A.nnz)}


def traffic_for(kernel):
    """DRAM bytes (read + write) of one launch of `kernel` (an ILU/ILUB application
    or an SpMV of a named workload) from ncu, as recorded in profiles/traffic.json
    with the command that measured it."""
    try:
        with open(TRAFFIC_JSON) as f:
            v = json.load(f).get(kernel)
        return int(v["bytes"]) if isinstance(v, dict) else None
    except (OSError, ValueError, KeyError, TypeError):
        return None


def cpu_solve(port, Ar, Lf, Uf, nc, sc, b, eps, m, threads):
    import oracle
    port.set_threads(threads)
    t0 = time.perf_counter()
    x, it, res, conv = port.solve("gmres", Ar, b, L=Lf, U=Uf, pc=oracle.PC_ILU_ABMC, cptr=sc, cnum=nc, bsize=16,
                                  outer=10000 // m, m=m, eps=eps, nrm_b=float(np.linalg.norm(b)))
    ms = (time.perf_counter() - t0) * 1e3
    port.set_threads(1)
    return ms, it, x


def _mean(xs):
    return sum(xs) / len(xs)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _timed(fn, steps, reset):
    """One untimed warm-up, then `steps` timed solves (device time on the
    library's stream); the last result is returned with the mean."""
    out = []
    for i in range(steps + 1):
        reset()
        r = fn()
        if i:
            out.append(r)
    return _mean([r.solve_ms for r in out]), out[-1]


def _kernel(sy, op, hbm, reps=10):
    ms, by = sy.time_op(op, reps)
    gbs = by / (ms * 1e-3) / 1e9 if ms > 0 else float("nan")
    return {"ms": round(ms, 4), "bytes": int(by), "gbs": round(gbs, 1), "frac": round(gbs / hbm, 4)}


def leg_bicgstab(sysm, Ar, b, nb, steps):
    """FP64 ABMC-ILU(0) BiCGStab on the headline system
    (include/senk_bicgstab.hpp:107-196; ABMC sweeps as for GMRES)."""
    ms, r = _timed(lambda: sysm.bicgstab(nb, 10000, 1e-8), steps, sysm.zero_x)
    x = sysm.get_x()
    return {"ms": ms, "iterations": r.iters, "converged": bool(r.converged),
            "true_residual": float(np.linalg.norm(b - Ar.matvec(x)) / nb), "dtype": "f64"}


def leg_c1(steps, with_cpu):
    """2D 5-point Poisson 128^2 (N = 16,384), b = A*1, ILU(0)-GMRES(30) to 1e-8 in
    natural order (level-set sweeps) and in ABMC order (bsize 16): warm GPU solves
    beside the CPU restatement of the reference on all host cores."""
    import oracle
    from senk_gb300 import lib as L
    from senk_gb300 import problems as P
    from senk_gb300 import setup as S
    from senk_gb300 import solver as SV
    A = P.poisson2d(128)
    b = A.matvec(np.ones(A.n))
    nb = float(np.linalg.norm(b))
    out = {"workload": "poisson2d 128^2, b = A*1, ILU(0)-GMRES(30), eps 1e-8, x0=0", "N": A.n, "nnz": A.nnz}
    Lf, Uf, _ = S.Split(S.Ilu0(A), "L-DU", True)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    La, Ua, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    cases = {"natural": (A, Lf, Uf, L.PC_ILU, None, 0, 1, b), "abmc16": (Ar, La, Ua, L.PC_ILU_ABMC, sc, nc, 16, b[LP])}
    port = oracle.port(threads=os.cpu_count() or 1) if with_cpu else None
    for name, (M, Lx, Ux, pc, cp, cn, bs, rhs) in cases.items():
        sy = SV.System(M, Lx, Ux, pc, cp, cn, bs, m_max=30)
        try:
            sy.set_rhs(rhs)
            ms, r = _timed(lambda: sy.gmres(nb, 10000 // 30, 30, 1e-8), max(steps, 5), sy.zero_x)
            x = sy.get_x()
        finally:
            sy.close()
        row = {"ms": ms, "iterations": r.iters, "true_residual": float(np.linalg.norm(rhs - M.matvec(x)) / nb),
               "us_per_iteration": 1e3 * ms / max(r.iters, 1)}
        if port is not None:
            opc = oracle.PC_ILU if pc == L.PC_ILU else oracle.PC_ILU_ABMC
            times, it = [], None
            for i in range(4):
                t0 = time.perf_counter()
                _, it, _, _ = port.solve("gmres", M, rhs, L=Lx, U=Ux, pc=opc, cptr=cp, cnum=cn, bsize=bs,
                                         outer=10000 // 30, m=30, eps=1e-8, nrm_b=nb)
                if i:
                    times.append((time.perf_counter() - t0) * 1e3)
            row["cpu_ms"] = _mean(times)
            row["cpu_iterations"] = it
            row["cpu_cores"] = os.cpu_count() or 1
        out[name] = row
    if port is not None:
        port.set_threads(1)
    return out


def leg_c3(n, steps, hbm, with_cpu):
    """Variable-coefficient diffusion n^3 (face coefficients exp of a Gaussian
    random field, sigma 1.5, correlation length 8), x_true ~ N(0,1): plain FP64
    ABMC-ILU(0)-GMRES(50) against FP64-outer GMRES-IR with FP32 factors, sweeps,
    inner SpMV and basis, both to 1e-10 FP64 true residual."""
    import oracle
    from senk_gb300 import lib as L
    from senk_gb300 import problems as P
    from senk_gb300 import setup as S
    from senk_gb300 import solver as SV
    t0 = time.perf_counter()
    A = P.vardiff3d(n, 1.5, 8.0, 0)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    Lf, Uf, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    b = Ar.matvec(P.normal_solution(A.n, 1)[LP])
    nb = float(np.linalg.norm(b))
    setup_s = time.perf_counter() - t0
    sy = SV.System(Ar, Lf, Uf, L.PC_ILU_ABMC, sc, nc, 16, m_max=50, mixed=1)
    try:
        sy.set_rhs(b)
        pms, rp = _timed(lambda: sy.gmres(nb, 10000 // 50, 50, 1e-10), steps, sy.zero_x)
        xp = sy.get_x()
        mms, rm = _timed(lambda: sy.gmres_ir(nb, 30, 50, 1e-10, 1e-4, 2), steps, sy.zero_x)
        xm = sy.get_x()
        kern = {"ilu_apply_f32": _kernel(sy, L.OP_INNER + L.OP_PRECOND, hbm),
                "ilu_apply_f64": _kernel(sy, L.OP_PRECOND, hbm),
                "spmv_f32": _kernel(sy, L.OP_INNER + L.OP_SPMV, hbm),
                "spmv_f64": _kernel(sy, L.OP_SPMV, hbm)}
    finally:
        sy.close()
    out = {"workload": f"vardiff3d {n}^3, sigma 1.5, corr 8, seed 0, ABMC bsize 16, ILU(0), GMRES(50), eps 1e-10",
           "N": Ar.n, "nnz": Ar.nnz, "colours": nc, "setup_s": round(setup_s, 1),
           "plain_fp64": {"ms": pms, "iterations": rp.iters, "converged": bool(rp.converged),
                          "true_residual": float(np.linalg.norm(b - Ar.matvec(xp)) / nb)},
           "gmres_ir": {"ms": mms, "iterations": rm.iters, "outer_steps": rm.cycles, "converged": bool(rm.converged),
                        "true_residual": float(np.linalg.norm(b - Ar.matvec(xm)) / nb),
                        "rel_err_vs_plain_fp64": _rel(xm, xp)},
           "kernels": kern,
           "roofline": dict(kernel="ILU(0) application, FP32 factors", bound="hbm", peak=hbm, unit="GB/s",
                            achieved=kern["ilu_apply_f32"]["gbs"], frac=kern["ilu_apply_f32"]["frac"],
                            traffic=traffic_for(f"ilu_apply_f32_vardiff{n}"))}
    if with_cpu:
        # one restart cycle (50 iterations) of the CPU restatement on all host cores
        port = oracle.port(threads=os.cpu_count() or 1)
        t0 = time.perf_counter()
        port.solve("gmres", Ar, b, L=Lf, U=Uf, pc=oracle.PC_ILU_ABMC, cptr=sc, cnum=nc, bsize=16, outer=1, m=50,
                   eps=1e-10, nrm_b=nb)
        cyc = (time.perf_counter() - t0) * 1e3
        port.set_threads(1)
        out["cpu_baseline"] = {"ms_per_50_iterations": cyc, "est_full_solve_ms": cyc * rp.iters / 50,
                               "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": "one GMRES(50) restart cycle of the FP64 solve, scaled to the GPU's "
                                         "iteration count"}
    return out


def leg_c4(n, steps, hbm, with_cpu):
    """Block-3x3 27-point system on n^3 nodes (dense 3x3 blocks, off-diagonal
    entries U(-1,0), SPD diagonal blocks with block dominance 1.1), ABMC on the
    node graph (4 nodes = 12 rows per block), ILUB(3x3): FP64 GCR(20) against
    FP64-outer GCR-IR with FP32 ILUB, inner SpMV and vectors, both to 1e-8."""
    import oracle
    from senk_gb300 import lib as L
    from senk_gb300 import problems as P
    from senk_gb300 import setup as S
    from senk_gb300 import solver as SV
    t0 = time.perf_counter()
    A = P.block27(n, seed=0)
    G = P.block27_node_graph(n)
    nc, sc, LPn, _ = S.GetABMCPermutation(G.cind, G.rptr, G.n, 4, False, "connect")
    LP, RP = P.expand_node_permutation(LPn, 3)
    Ar = S.Reordering(A, LP, RP)
    del A
    Lf, Uf, _ = S.Split(S.Ilu0(S.AllocBlockZero(Ar, 3, 3)), "L-DU", True)
    bl, bu = S.Csr2Bcsr(Lf, 3, 3), S.Csr2Bcsr(Uf, 3, 3)
    del Lf, Uf
    b = Ar.matvec(P.uniform_solution(Ar.n, 2)[LP])
    nb = float(np.linalg.norm(b))
    setup_s = time.perf_counter() - t0
    sy = SV.System(Ar, bl, bu, L.PC_ILUB_ABMC, sc, nc, 12, m_max=0, block=(3, 3), mixed=1)
    try:
        sy.set_rhs(b)
        pms, rp = _timed(lambda: sy.gcr(nb, 500, 20, 1e-8), steps, sy.zero_x)
        xp = sy.get_x()
        mms, rm = _timed(lambda: sy.gcr_ir(nb, 30, 20, 1e-8, 1e-4, 5), steps, sy.zero_x)
        xm = sy.get_x()
        kern = {"ilub_apply_f32": _kernel(sy, L.OP_INNER + L.OP_PRECOND, hbm),
                "ilub_apply_f64": _kernel(sy, L.OP_PRECOND, hbm),
                "spmv_f32": _kernel(sy, L.OP_INNER + L.OP_SPMV, hbm),
                "spmv_f64": _kernel(sy, L.OP_SPMV, hbm)}
    finally:
        sy.close()
    out = {"workload": f"block27 {n}^3 nodes, 3x3 blocks, ABMC on nodes (4 per block), ILUB(3x3), GCR(20), "
                       "eps 1e-8", "N": Ar.n, "nnz": Ar.nnz, "colours": nc, "setup_s": round(setup_s, 1),
           "plain_fp64": {"ms": pms, "iterations": rp.iters, "converged": bool(rp.converged),
                          "true_residual": float(np.linalg.norm(b - Ar.matvec(xp)) / nb)},
           "gcr_ir": {"ms": mms, "iterations": rm.iters, "outer_steps": rm.cycles, "converged": bool(rm.converged),
                      "true_residual": float(np.linalg.norm(b - Ar.matvec(xm)) / nb),
                      "rel_err_vs_plain_fp64": _rel(xm, xp)},
           "kernels": kern,
           "roofline": dict(kernel="ILUB(3x3) application, FP32 factors", bound="hbm", peak=hbm, unit="GB/s",
                            achieved=kern["ilub_apply_f32"]["gbs"], frac=kern["ilub_apply_f32"]["frac"],
                            traffic=traffic_for(f"ilub_apply_f32_block27_{n}"))}
    if with_cpu:
        port = oracle.port(threads=os.cpu_count() or 1)
        t0 = time.perf_counter()
        port.solve("gcr", Ar, b, L=bl, U=bu, pc=oracle.PC_ILUB_ABMC, cptr=sc, cnum=nc, bsize=12, bnl=3, bnw=3,
                   outer=1, m=20, eps=1e-8, nrm_b=nb)
        cyc = (time.perf_counter() - t0) * 1e3
        port.set_threads(1)
        out["cpu_baseline"] = {"ms_per_20_iterations": cyc, "est_full_solve_ms": cyc * max(rp.iters, 20) / 20,
                               "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": "one GCR(20) restart cycle of the FP64 solve, scaled to the GPU's "
                                         "iteration count"}
    return out


def run_reference(args, rank):
    """The reference's CPU algorithm (the C restatement in oracle/, OpenMP over all
    host cores) on the same workload."""
    if rank != 0:
        return
    import oracle
    port = oracle.port()
    threads = os.cpu_count() or 1
    A, xt = problem(args.n)
    Ar, Lf, Uf, nc, sc, b = setup_oracle(port, A, xt)
    for _ in range(args.warmup):
        cpu_solve(port, Ar, Lf, Uf, nc, sc, b, args.eps, args.m, threads)
    times, its = [], []
    for _ in range(args.steps):
        ms, it, x = cpu_solve(port, Ar, Lf, Uf, nc, sc, b, args.eps, args.m, threads)
        times.append(ms)
        its.append(it)
    v = sum(times) / len(times)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(args.n), "N": A.n, "nnz": A.nnz, "colours": nc,
                       "iterations": its[-1]},
            "cpu_baseline": {"value": v, "unit": "ms", "cores": threads, "kind": "port",
                             "sample": "full solves of the workload (oracle C restatement of the reference, "
                                       "OpenMP, reference compiled headers are not available on this host)"},
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world):
    import torch
    from senk_gb300 import lib as L
    from senk_gb300 import solver as SV
    local = int(os.environ.get("LOCAL_RANK", 0))
    L.check("set_device", L.lib().senk_set_device(local))
    A, xt = problem(args.n)
    Ar, Lf, Uf, nc, sc, b = setup_gpu(A, xt)
    nb = float(np.linalg.norm(b))
    orth = {"cgs2": L.ORTH_CGS2, "cgs": L.ORTH_CGS, "mgs": L.ORTH_MGS}[args.orth]
    spmv = {"auto": L.SPMV_AUTO, "csr": L.SPMV_CSR, "sell": L.SPMV_SELL, "sell_sigma": L.SPMV_SELL_SIGMA}[args.spmv]
    sweep = {"auto": L.SWEEP_AUTO, "colours": L.SWEEP_COLOURS, "dataflow": L.SWEEP_DATAFLOW,
             "compact": L.SWEEP_COMPACT, "persistent": L.SWEEP_PERSISTENT, "wide": L.SWEEP_WIDE, "rows": L.SWEEP_ROWS,
             "rows_wide": L.SWEEP_ROWS_WIDE}[args.sweep]
    outer = 10000 // args.m
    ir_outer = 20
    sysm = SV.System(Ar, Lf, Uf, L.PC_ILU_ABMC, sc, nc, 16, m_max=args.m, mixed=True, orth=orth, spmv=spmv,
                     sweep=sweep)
    sysm.set_rhs(b)
    do_mixed, do_plain = args.only in ("both", "mixed"), args.only in ("both", "plain")
    mixed = lambda: sysm.gmres_ir(nb, ir_outer, args.m, args.eps, args.inner_tol, args.inner_cycles)
    plain = lambda: sysm.gmres(nb, outer, args.m, args.eps)
    for _ in range(args.warmup):
        if do_mixed:
            sysm.zero_x()
            mixed()
        if do_plain:
            sysm.zero_x()
            plain()
    barrier(world)
    res_m, res_p = [], []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            if do_mixed:
                sysm.zero_x()
                res_m.append(mixed())
    if do_mixed:
        x_m = sysm.get_x()
        true_m = float(np.linalg.norm(b - Ar.matvec(x_m)) / nb)
    for _ in range(args.steps):
        if do_plain:
            sysm.zero_x()
            res_p.append(plain())
    if do_plain:
        x_p = sysm.get_x()
        true_p = float(np.linalg.norm(b - Ar.matvec(x_p)) / nb)
    barrier(world)
    legs = [x for x in args.legs.split(",") if x]
    bicg = leg_bicgstab(sysm, Ar, b, nb, args.leg_steps) if "bicgstab" in legs and rank == 0 else None
    mean = lambda rs: sum(r.solve_ms for r in rs) / len(rs)
    hbm, peak_kind = peaks()
    reps = 0 if args.no_kernels else 20
    timed = lambda op: sysm.time_op(op, reps) if reps else (float("nan"), 0)
    gbs = lambda by, ms: by / (ms * 1e-3) / 1e9 if ms == ms and ms > 0 else float("nan")
    kern = {}
    for tag, base in (("f32", L.OP_INNER), ("f64", 0)):
        for name, op in (("ilu_apply", L.OP_PRECOND), ("sptrsv_l", L.OP_SWEEP_L), ("sptrsv_u", L.OP_SWEEP_U),
                         ("spmv", L.OP_SPMV), ("dot", L.OP_DOT)):
            ms, by = timed(base + op)
            kern[f"{name}_{tag}_ms"] = ms
            kern[f"{name}_{tag}_gbs"] = gbs(by, ms)
            kern[f"{name}_{tag}_bytes"] = by
    sysm.close()
    e2e = None
    if not args.no_e2e and do_mixed:
        e2e_ms, rr, cold = [], None, None
        # the caller's b and x in pinned host memory
        bh = torch.empty(Ar.n, dtype=torch.float64, pin_memory=True).numpy()
        xh = torch.empty(Ar.n, dtype=torch.float64, pin_memory=True).numpy()
        bh[:] = b
        for i in range(max(1, min(args.steps, 3)) + 1):  # the first call builds the device system
            xh[:] = 0.0
            t0 = time.perf_counter()
            rr = SV.AbmcIluGmresIr(Ar.val, Ar.cind, Ar.rptr, Lf.val, Lf.cind, Lf.rptr, Uf.val, Uf.cind, Uf.rptr, sc,
                                   nc, 16, bh, xh, nb, ir_outer, args.m, Ar.n, args.eps, args.inner_tol,
                                   args.inner_cycles, orth=orth, spmv=spmv, sweep=sweep)
            ms = (time.perf_counter() - t0) * 1e3
            if i > 0:
                e2e_ms.append(ms)
            else:
                cold = {"ms": ms, "h2d_bytes": int(rr.h2d_bytes)}
        e2e = {"value": allmax(world, sum(e2e_ms) / len(e2e_ms)), "unit": "ms",
               "h2d_bytes_per_step": int(rr.h2d_bytes), "d2h_bytes_per_step": int(rr.d2h_bytes),
               "steps": len(e2e_ms), "iterations": rr.iters, "first_call": cold,
               "note": "drop-in C ABI call senk_abmc_ilu_gmres_ir_d with host arrays (b and x pinned), wall "
                       "clock; A and the factors stay on the device between calls (content-hashed every call), "
                       "so a step uploads b and x0 and reads x back; first_call includes building the device "
                       "system"}
    learned = None
    if not args.no_learned and "learned" in legs and rank == 0:
        learned = learned_leg()
    with_cpu = rank == 0 and world == 1 and not args.no_cpu_baseline
    extra = {}
    if rank == 0:
        if "c1" in legs:
            extra["c1"] = leg_c1(args.leg_steps, with_cpu)
        if "c3" in legs:
            extra["c3"] = leg_c3(args.c3_n, args.leg_steps, peaks()[0], with_cpu)
        if "c4" in legs:
            extra["c4"] = leg_c4(args.c4_n, args.leg_steps, peaks()[0], with_cpu)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        port = oracle.port()
        threads = os.cpu_count() or 1
        cms, cit, _ = cpu_solve(port, Ar, Lf, Uf, nc, sc, b, args.eps, args.m, threads)
        cpu = {"value": cms, "unit": "ms", "cores": threads, "kind": "port",
               "sample": f"one full FP64 solve of the workload ({cit} iterations), oracle C restatement of the "
                         "reference with OpenMP"}
    if rank != 0:
        return
    value = allmax(world, mean(res_m)) if do_mixed else allmax(world, mean(res_p))
    rm = res_m[-1] if do_mixed else None
    rp = res_p[-1] if do_plain else None
    dom = "ilu_apply_f32" if do_mixed else "ilu_apply_f64"
    line = {
        "metric": METRIC, "value": value, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if do_mixed else "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.n), "N": Ar.n, "nnz": Ar.nnz, "colours": nc,
                   "orth": args.orth, "spmv": args.spmv, "sweep": args.sweep, "inner_tol": args.inner_tol,
                   "inner_cycles": args.inner_cycles,
                   "iterations": rm.iters if rm else rp.iters,
                   "outer_steps": rm.cycles if rm else None,
                   "true_residual": true_m if rm else true_p,
                   "l2": "inputs larger than L2 (A, L, U and the Krylov bases, about 1.2 GB)",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "plain_fp64": None if rp is None else {"ms": allmax(world, mean(res_p)), "iterations": rp.iters,
                                               "cycles": rp.cycles, "implicit_residual": rp.res,
                                               "true_residual": true_p},
        "mixed_rel_err_vs_plain_fp64": _rel(x_m, x_p) if (rm and rp) else None,
        "bicgstab": bicg,
        "e2e": e2e,
        "gpu_launches": int(sum(x.launches for x in (res_m if do_mixed else res_p))),
        "roofline": {"kernel": "ILU(0) application (ABMC L and U sweeps, all colours), "
                               + ("FP32 factors" if do_mixed else "FP64"),
                     "bound": "hbm", "achieved": kern[dom + "_gbs"], "peak": hbm, "unit": "GB/s",
                     "frac": kern[dom + "_gbs"] / hbm, "peak_source": peak_kind, "traffic": traffic_for(dom),
                     "bytes_per_launch": kern[dom + "_bytes"], "ms_per_launch": kern[dom + "_ms"]},
        "kernels": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in kern.items()},
        "cpu_baseline": cpu,
        "learned": learned,
        **extra,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


_pg = None


def init_dist():
    global _pg
    world = int(os.environ.get("WORLD_SIZE", 1))
    rank = int(os.environ.get("RANK", 0))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        _pg = dist
    return rank, world


def barrier(world):
    if world > 1 and _pg is not None:
        _pg.barrier()


def allmax(world, v):
    if world > 1 and _pg is not None:
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        _pg.all_reduce(t, op=_pg.ReduceOp.MAX)
        return float(t.item())
    return v


def main():
    args = parse()
    rank, world = init_dist()
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
