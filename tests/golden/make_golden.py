"""Regenerate the golden fixtures from the reference itself.

Runs SenK's own headers (compiled by ``oracle/Makefile`` into
``oracle/_ref/libsenk_ref.so``) on seeded synthetic inputs and stores what they
produce: colouring/permutation arrays, ILU factors, kernel outputs and solver
iteration counts/residuals as printed by the reference.  The fixtures travel with
the repository, so the CPU restatement and the CUDA path can be checked against
the reference on machines where its sources are absent.

    python tests/golden/make_golden.py      # needs the reference sources
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from senk_gb300 import problems as P  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def solve_ref(R, name, *args):
    txt = R.solve_text(name, *args)
    p = oracle.parse_solver_stdout(txt)
    return {"iters": p["iters"], "res": p["res"], "converged": p["converged"]}


def c1_record(R):
    """2D Poisson 128^2, b = A*1, x0 = 0: every solver family at 1e-8."""
    A = P.poisson2d(128)
    N = A.n
    b = A.matvec(np.ones(N))
    nb = float(np.sqrt(np.dot(b, b)))
    rec = {"N": N, "nnz": A.nnz, "eps": 1e-8}
    F = R.ilu0(A)
    L, U, _ = R.split(F, "L-DU", True)
    rec["ilu_natural"] = {"L_sha": sha(L.val), "U_sha": sha(U.val),
                          "Lpat_sha": sha(np.concatenate([L.rptr, L.cind])),
                          "Upat_sha": sha(np.concatenate([U.rptr, U.cind]))}
    x = np.zeros(N)
    rec["Gmresm_m30"] = solve_ref(R, "gmres_d", A.val, A.cind, A.rptr, b, x, nb, 10000 // 30, 30, N, 1e-8)
    x = np.zeros(N)
    rec["IluGmresm_m30"] = solve_ref(R, "ilu_gmres_d", A.val, A.cind, A.rptr, L.val, L.cind, L.rptr,
                                     U.val, U.cind, U.rptr, b, x, nb, 10000 // 30, 30, N, 1e-8)
    x = np.zeros(N)
    rec["IluBicgstab"] = solve_ref(R, "ilu_bicgstab_d", A.val, A.cind, A.rptr, L.val, L.cind, L.rptr,
                                   U.val, U.cind, U.rptr, b, x, nb, 10000, N, 1e-8)
    x = np.zeros(N)
    rec["IluGcrm_m20"] = solve_ref(R, "ilu_gcr_d", A.val, A.cind, A.rptr, L.val, L.cind, L.rptr,
                                   U.val, U.cind, U.rptr, b, x, nb, 10000 // 20, 20, N, 1e-8)
    x = np.zeros(N)
    rec["Bicgstab"] = solve_ref(R, "bicgstab_d", A.val, A.cind, A.rptr, b, x, nb, 10000, N, 1e-8)

    # ABMC (bsize 16, "connect", isSym=false) and AMC orderings of the same system
    nc, sc, LP, RP = R.abmc_permutation(A.cind, A.rptr, N, 16, False, "connect")
    Ar = R.reordering(A, LP, RP)
    br = b[LP]
    Fr = R.ilu0(Ar)
    Lr, Ur, _ = R.split(Fr, "L-DU", True)
    x = np.zeros(N)
    rec["abmc16"] = {"num_color": nc, "size_color": sc.tolist(), "LP_sha": sha(LP), "RP_sha": sha(RP),
                     "A_sha": sha(np.concatenate([Ar.rptr, Ar.cind])), "Aval_sha": sha(Ar.val),
                     "L_sha": sha(Lr.val), "U_sha": sha(Ur.val)}
    rec["AbmcIluGmresm_m30"] = solve_ref(R, "abmc_ilu_gmres_d", Ar.val, Ar.cind, Ar.rptr, Lr.val, Lr.cind,
                                         Lr.rptr, Ur.val, Ur.cind, Ur.rptr, sc, nc, 16, br, x, nb,
                                         10000 // 30, 30, N, 1e-8)
    nc2, sc2, LP2, RP2 = R.amc_permutation(A.cind, A.rptr, N, False)
    Aa = R.reordering(A, LP2, RP2)
    Fa = R.ilu0(Aa)
    La, Ua, _ = R.split(Fa, "L-DU", True)
    x = np.zeros(N)
    rec["amc"] = {"num_color": nc2, "size_color": sc2.tolist(), "LP_sha": sha(LP2)}
    rec["AmcIluGmresm_m30"] = solve_ref(R, "amc_ilu_gmres_d", Aa.val, Aa.cind, Aa.rptr, La.val, La.cind,
                                        La.rptr, Ua.val, Ua.cind, Ua.rptr, sc2, nc2, b[LP2], x, nb,
                                        10000 // 30, 30, N, 1e-8)
    # ILUB 8x1 (AllocBlockZero + Ilu0 + Split + Csr2Bcsr), natural order
    Ab = R.alloc_block_zero(A, 8, 1)
    Fb = R.ilu0(Ab)
    Lb, Ub, _ = R.split(Fb, "L-DU", True)
    bl = R.csr2bcsr(Lb, 8, 1)
    bu = R.csr2bcsr(Ub, 8, 1)
    x = np.zeros(N)
    rec["IlubGmresm_8x1_m30"] = solve_ref(R, "ilub_gmres_d", A.val, A.cind, A.rptr, *bl, *bu, b, x, nb,
                                          10000 // 30, 30, N, 1e-8, 8, 1)
    rec["ilub_8x1"] = {"nnz": Ab.nnz, "pattern_sha": sha(np.concatenate([Ab.rptr, Ab.cind])),
                       "Lb_sha": sha(bl[0]), "Ub_sha": sha(bu[0])}
    x = np.zeros(N)
    rec["IlubGcrm_8x1_m20"] = solve_ref(R, "ilub_gcr_d", A.val, A.cind, A.rptr, *bl, *bu, b, x, nb,
                                        10000 // 20, 20, N, 1e-8, 8, 1)
    x = np.zeros(N)
    rec["IlubBicgstab_8x1"] = solve_ref(R, "ilub_bicgstab_d", A.val, A.cind, A.rptr, *bl, *bu, b, x, nb,
                                        10000, N, 1e-8, 8, 1)
    # ILUB 2x2: blocks two columns wide
    Ab2 = R.alloc_block_zero(A, 2, 2)
    Lb2, Ub2, _ = R.split(R.ilu0(Ab2), "L-DU", True)
    x = np.zeros(N)
    rec["IlubGmresm_2x2_m30"] = solve_ref(R, "ilub_gmres_d", A.val, A.cind, A.rptr, *R.csr2bcsr(Lb2, 2, 2),
                                          *R.csr2bcsr(Ub2, 2, 2), b, x, nb, 10000 // 30, 30, N, 1e-8, 2, 2)
    # ABMC (bsize 16) + ILUB 8x1 on the reordered system (the reference's main.cpp flow)
    Abr = R.alloc_block_zero(Ar, 8, 1)
    Lbr, Ubr, _ = R.split(R.ilu0(Abr), "L-DU", True)
    x = np.zeros(N)
    rec["AbmcIlubGmresm_8x1_m30"] = solve_ref(R, "abmc_ilub_gmres_d", Ar.val, Ar.cind, Ar.rptr,
                                              *R.csr2bcsr(Lbr, 8, 1), *R.csr2bcsr(Ubr, 8, 1), sc, nc, 16,
                                              br, x, nb, 10000 // 30, 30, N, 1e-8, 8, 1)
    # block Jacobi, 16 blocks: ILU(0) of RemoveOffDiagonal(A)
    Aj = R.remove_off_diagonal(A, 16)
    Lj, Uj, _ = R.split(R.ilu0(Aj), "L-DU", True)
    x = np.zeros(N)
    rec["BjIluGmresm_16_m30"] = solve_ref(R, "bj_ilu_gmres_d", A.val, A.cind, A.rptr, Lj.val, Lj.cind, Lj.rptr,
                                          Uj.val, Uj.cind, Uj.rptr, 16, b, x, nb, 10000 // 30, 30, N, 1e-8)
    rec["bj16"] = {"nnz": Aj.nnz, "pattern_sha": sha(np.concatenate([Aj.rptr, Aj.cind]))}
    # unpreconditioned GCR(20) and GMRES(30) on the 2x2 BCSR form of A
    x = np.zeros(N)
    rec["Gcrm_m20"] = solve_ref(R, "gcr_d", A.val, A.cind, A.rptr, b, x, nb, 10000 // 20, 20, N, 1e-8)
    x = np.zeros(N)
    rec["BcsrGmresm_2x2_m30"] = solve_ref(R, "bcsr_gmres_d", *R.csr2bcsr(A, 2, 2), b, x, nb, 10000 // 30, 30, N,
                                          1e-8, 2, 2)
    # FP32 ILU-GMRES at 1e-6 (the reference instantiated with T=float)
    Af = A.astype(np.float32)
    xf = np.zeros(N, np.float32)
    rec["IluGmresm_float_m30"] = solve_ref(
        R, "ilu_gmres_s", Af.val, Af.cind, Af.rptr, L.val.astype(np.float32), L.cind, L.rptr,
        U.val.astype(np.float32), U.cind, U.rptr, b.astype(np.float32), xf,
        ctypes.c_float(np.sqrt(np.dot(b, b))), 10000 // 30, 30, N, ctypes.c_float(1e-6))
    return rec


def small_arrays(R):
    """16^3 convection-diffusion: arrays small enough to store whole."""
    A = P.convdiff3d(16, 0.5)
    N = A.n
    xt = P.uniform_solution(N, 0)
    nc, sc, LP, RP = R.abmc_permutation(A.cind, A.rptr, N, 16, False, "connect")
    Ar = R.reordering(A, LP, RP)
    F = R.ilu0(Ar)
    L, U, _ = R.split(F, "L-DU", True)
    rng = np.random.default_rng(7)
    v = rng.uniform(-1, 1, N)
    y_spmv = R.spmv_csr(Ar, v)
    t = R.sptrsv(L, v, False, sc, nc, 16)
    y_ilu_abmc = R.sptrsv(U, t, True, sc, nc, 16)
    t = R.sptrsv(L, v, False)
    y_ilu_seq = R.sptrsv(U, t, True)
    b = Ar.matvec(xt[LP])
    nb = float(np.sqrt(np.dot(b, b)))
    x = np.zeros(N)
    g = solve_ref(R, "abmc_ilu_gmres_d", Ar.val, Ar.cind, Ar.rptr, L.val, L.cind, L.rptr, U.val, U.cind,
                  U.rptr, sc, nc, 16, b, x, nb, 100, 30, N, 1e-8)
    x2 = np.zeros(N)
    h = solve_ref(R, "ilu_bicgstab_d", Ar.val, Ar.cind, Ar.rptr, L.val, L.cind, L.rptr, U.val, U.cind,
                  U.rptr, b, x2, nb, 1000, N, 1e-8)
    # ILUB 8x1 on the reordered system: BCSR factors and both sweep schedules
    Lb, Ub, _ = R.split(R.ilu0(R.alloc_block_zero(Ar, 8, 1)), "L-DU", True)
    bl, bu = R.csr2bcsr(Lb, 8, 1), R.csr2bcsr(Ub, 8, 1)
    y_ilub_seq = R.ilub_apply(bl, bu, v, 8, 1)
    y_ilub_abmc = R.ilub_apply(bl, bu, v, 8, 1, sc, nc, 16)
    ilub = dict(Lb_val=bl[0], Lb_cind=bl[1], Lb_rptr=bl[2], Ub_val=bu[0], Ub_cind=bu[1], Ub_rptr=bu[2],
                y_ilub_seq=y_ilub_seq, y_ilub_abmc=y_ilub_abmc)
    arrays = dict(**ilub, A_val=A.val, A_cind=A.cind, A_rptr=A.rptr, LP=LP, RP=RP, size_color=sc,
                  Ar_val=Ar.val, Ar_cind=Ar.cind, Ar_rptr=Ar.rptr, L_val=L.val, L_cind=L.cind,
                  L_rptr=L.rptr, U_val=U.val, U_cind=U.cind, U_rptr=U.rptr, v=v, y_spmv=y_spmv,
                  y_ilu_abmc=y_ilu_abmc, y_ilu_seq=y_ilu_seq, b=b, x_gmres=x, x_bicgstab=x2)
    meta = {"num_color": nc, "AbmcIluGmresm_m30": g, "IluBicgstab": h}
    return arrays, meta


def main():
    R = oracle.ref()
    if R is None:
        raise SystemExit("the reference sources are needed to regenerate the fixtures")
    rec = {"c1": c1_record(R)}
    arrays, meta = small_arrays(R)
    rec["convdiff16"] = meta
    np.savez_compressed(os.path.join(OUT, "convdiff16.npz"), **arrays)
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(rec, f, indent=1, sort_keys=True)
    print(json.dumps(rec, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
