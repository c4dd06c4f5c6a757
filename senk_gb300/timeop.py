"""Time one operation of the solve path, with CUDA events on the system's stream,
on one of the benchmarked systems:

    python -m senk_gb300.timeop --op precond --dtype f32 --n 128 --reps 50

Problems: convdiff (3D convection-diffusion, Pe 0.5, ABMC bsize 16, ILU(0); the
headline system), vardiff (variable-coefficient diffusion, sigma 1.5, correlation
length 8, seed 0, ABMC bsize 16, ILU(0)), block27 (3x3 blocks on n^3 nodes, ABMC
on the node graph with 4 nodes per block, ILUB(3x3)), poisson2d (5-point n^2,
ILU(0) in the natural order, or ABMC bsize 16 with --order abmc).

Ops: spmv, precond (L then U sweeps, all colours), sweep_l, sweep_u, dot,
multidot and update (the Arnoldi step over 16 basis vectors). Prints
one JSON line (mean ms per run, algorithmic bytes, GB/s). The first run is
untimed, so a profiler that captures the first launches of a kernel sees one
complete run.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import lib as L
from . import problems as P
from . import setup as S
from .solver import System

OPS = {"spmv": L.OP_SPMV, "precond": L.OP_PRECOND, "sweep_l": L.OP_SWEEP_L, "sweep_u": L.OP_SWEEP_U,
       "dot": L.OP_DOT, "multidot": L.OP_MULTIDOT, "update": L.OP_UPDATE}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="precond", choices=sorted(OPS))
    ap.add_argument("--dtype", default="f32", choices=["f32", "f64"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--reps", type=int, default=50)
    ap.add_argument("--sweep", default="auto",
                    choices=["auto", "colours", "dataflow", "compact", "persistent", "wide", "rows", "rows_wide"])
    ap.add_argument("--problem", default="convdiff", choices=["convdiff", "vardiff", "block27", "poisson2d"])
    ap.add_argument("--order", default="abmc", choices=["abmc", "natural"], help="poisson2d only")
    args = ap.parse_args(argv)
    dt = np.float32 if args.dtype == "f32" else np.float64
    sweep = {"auto": L.SWEEP_AUTO, "colours": L.SWEEP_COLOURS, "dataflow": L.SWEEP_DATAFLOW,
             "compact": L.SWEEP_COMPACT, "persistent": L.SWEEP_PERSISTENT, "wide": L.SWEEP_WIDE, "rows": L.SWEEP_ROWS,
             "rows_wide": L.SWEEP_ROWS_WIDE}[args.sweep]
    if args.problem == "block27":
        A, G = P.block27(args.n, seed=0), P.block27_node_graph(args.n)
        nc, sc, LPn, _ = S.GetABMCPermutation(G.cind, G.rptr, G.n, 4, False, "connect")
        LP, RP = P.expand_node_permutation(LPn, 3)
        Ar = S.Reordering(A, LP, RP)
        del A
        Lf, Uf, _ = S.Split(S.Ilu0(S.AllocBlockZero(Ar, 3, 3)), "L-DU", True)
        sy = System(Ar, S.Csr2Bcsr(Lf, 3, 3), S.Csr2Bcsr(Uf, 3, 3), L.PC_ILUB_ABMC, sc, nc, 12, dtype=dt,
                    m_max=1, block=(3, 3), sweep=sweep)
    elif args.problem == "poisson2d" and args.order == "natural":
        A = P.poisson2d(args.n)
        Ar, nc = A, 0
        Lf, Uf, _ = S.Split(S.Ilu0(A), "L-DU", True)
        sy = System(A, Lf, Uf, L.PC_ILU, None, 0, 1, dtype=dt, m_max=1, sweep=sweep)
    else:
        A = {"convdiff": lambda: P.convdiff3d(args.n, 0.5), "vardiff": lambda: P.vardiff3d(args.n, 1.5, 8.0, 0),
             "poisson2d": lambda: P.poisson2d(args.n)}[args.problem]()
        nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
        Ar = S.Reordering(A, LP, RP)
        Lf, Uf, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
        sy = System(Ar, Lf, Uf, L.PC_ILU_ABMC, sc, nc, 16, dtype=dt, m_max=1, sweep=sweep)
    ms, by = sy.time_op(OPS[args.op], args.reps)
    sy.close()
    print(json.dumps(dict(op=args.op, problem=args.problem, order=args.order, dtype=args.dtype, sweep=args.sweep,
                          n=args.n, N=Ar.n, colours=nc, ms=ms, bytes=by, gbs=by / ms / 1e6 if ms > 0 else None)))


if __name__ == "__main__":
    main()
