"""Time one operation of the solve path on the 3D convection-diffusion workload
(the benchmark's system), with CUDA events on the system's stream:

    python -m senk_gb300.timeop --op precond --dtype f32 --n 128 --reps 50

Ops: spmv, precond (L then U sweeps, all colours), sweep_l, sweep_u, dot. Prints
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
       "dot": L.OP_DOT}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="precond", choices=sorted(OPS))
    ap.add_argument("--dtype", default="f32", choices=["f32", "f64"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--reps", type=int, default=50)
    ap.add_argument("--sweep", default="auto", choices=["auto", "colours", "dataflow", "compact"])
    args = ap.parse_args(argv)
    A = P.convdiff3d(args.n, 0.5)
    nc, sc, LP, RP = S.GetABMCPermutation(A.cind, A.rptr, A.n, 16, False, "connect")
    Ar = S.Reordering(A, LP, RP)
    Lf, Uf, _ = S.Split(S.Ilu0(Ar), "L-DU", True)
    dt = np.float32 if args.dtype == "f32" else np.float64
    sweep = {"auto": L.SWEEP_AUTO, "colours": L.SWEEP_COLOURS, "dataflow": L.SWEEP_DATAFLOW,
             "compact": L.SWEEP_COMPACT}[args.sweep]
    sy = System(Ar, Lf, Uf, L.PC_ILU_ABMC, sc, nc, 16, dtype=dt, m_max=1, sweep=sweep)
    ms, by = sy.time_op(OPS[args.op], args.reps)
    sy.close()
    print(json.dumps(dict(op=args.op, dtype=args.dtype, sweep=args.sweep, n=args.n, N=Ar.n, colours=nc, ms=ms,
                          bytes=by,
                          gbs=by / ms / 1e6 if ms > 0 else None)))


if __name__ == "__main__":
    main()
