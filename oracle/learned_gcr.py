"""ORACLE — test infrastructure, not product code.

Per-iteration comparison of flexible GCR(m) with K = ILU(0) and with
K = ILU(0) + network, on the CPU: the network is the numpy restatement in
``oracle/mpnn.py`` (float64, no BF16 rounding), trained the way
``senk_gb300.learned.train`` trains the GPU network (residual-space loss, Adam,
global-norm clip 1, pairs from ILU(0)-GMRES(10) iterates after 1-4 restart
cycles); ILU(0) is ``port().ilu_apply``.

GCR here records the residual after every iteration. The reference's GCR
(``senk_gcr.hpp:93-161``, IluGcrm) tests convergence only at restarts, so its
iteration counts come in multiples of m and hide differences smaller than a
restart cycle; this history shows them.

    python -m oracle.learned_gcr --n 16 --train 16 --epochs 3 --lr 3e-4 [--step 1]
"""
from __future__ import annotations

import numpy as np

from . import PC_ILU_ABMC, port
from . import mpnn as M


def gmres_pairs(P, mb, cycles=(1, 2, 3, 4), m=10):
    """(r_k, e_k, ILU(r_k)) from ILU(0)-GMRES(m) iterates after the given
    numbers of restart cycles (x_0 = 0)."""
    out = []
    nb = float(np.linalg.norm(mb.b))
    for k in cycles:
        x, _, _, _ = P.solve("gmres", mb.A, mb.b, L=mb.L, U=mb.U, pc=PC_ILU_ABMC, cptr=mb.cptr, cnum=mb.cnum,
                             bsize=16, outer=k, m=m, eps=1e-14, nrm_b=nb)
        r = mb.b - mb.A.matvec(x)
        out.append((r, mb.x_true - x, P.ilu_apply(mb.L, mb.U, r, mb.cptr, mb.cnum, 16)))
    return out


def train(members, epochs=3, lr=3e-4, clip=1.0, seed=0):
    """Adam on the residual-space loss, one step per pair; returns (params, losses)."""
    P = port()
    prm = M.init_params(seed).astype(np.float64)
    m1 = np.zeros_like(prm)
    v1 = np.zeros_like(prm)
    t = 0
    losses = []
    for _ in range(epochs):
        for mb in members():
            g = M.Graph(mb.A.val, mb.A.cind, mb.A.rptr)
            for r, e, ilu in gmres_pairs(P, mb):
                loss, G = M.loss_grad(prm, g, r, ilu, e, rounding=False, mode=1)
                gn = float(np.linalg.norm(G))
                if gn > clip:
                    G = G * (clip / gn)
                t += 1
                m1 = 0.9 * m1 + 0.1 * G
                v1 = 0.999 * v1 + 0.001 * G * G
                prm -= lr * (m1 / (1 - 0.9 ** t)) / (np.sqrt(v1 / (1 - 0.999 ** t)) + 1e-8)
                losses.append(loss)
    return prm, losses


def gcr_history(A, b, K, m=20, iters=60):
    """Flexible GCR(m) from x = 0 (the steps of IluGcrm, senk_gcr.hpp:93-161,
    with K(r) in place of the ILU application): ||r_k|| / ||b|| for k = 0..iters."""
    x = np.zeros(A.n)
    r = np.array(b, np.float64)
    nb = float(np.linalg.norm(b))
    hist = [1.0]
    while len(hist) <= iters:
        Pd, AP, APn = [], [], []
        z = K(r)
        Az = A.matvec(z)
        Pd.append(z)
        AP.append(Az)
        APn.append(Az @ Az)
        for j in range(m):
            a = (AP[j] @ r) / APn[j]
            x += a * Pd[j]
            r -= a * AP[j]
            hist.append(float(np.linalg.norm(r)) / nb)
            if len(hist) > iters or j == m - 1:
                break
            z = K(r)
            Az = A.matvec(z)
            p, ap = z.copy(), Az.copy()
            for k in range(j + 1):
                beta = -(Az @ AP[k]) / APn[k]
                p += beta * Pd[k]
                ap += beta * AP[k]
            Pd.append(p)
            AP.append(ap)
            APn.append(ap @ ap)
    return np.array(hist)


def first_below(h, tol):
    return int(np.argmax(h < tol)) if (h < tol).any() else -1


def compare(prm, mb, m=20, iters=60, eps=1e-8, step=0):
    """Residual histories of GCR(m) with K = ILU and K = ILU + net on one system
    (step 1: the correction scaled by its least-squares step, mpnn.apply_step)."""
    P = port()
    g = M.Graph(mb.A.val, mb.A.cind, mb.A.rptr)

    def ilu(r):
        return P.ilu_apply(mb.L, mb.U, r, mb.cptr, mb.cnum, 16)

    h0 = gcr_history(mb.A, mb.b, ilu, m, iters)
    K = M.apply_step if step else M.apply
    h1 = gcr_history(mb.A, mb.b, lambda r: K(prm, g, r, ilu(r), rounding=False), m, iters)
    return dict(plain_iters=first_below(h0, eps), learned_iters=first_below(h1, eps),
                plain_res=[float(h0[i]) for i in range(0, iters + 1, 10)],
                learned_res=[float(h1[i]) for i in range(0, iters + 1, 10)])


def main(argv=None):
    import argparse
    import json

    from senk_gb300.learned import family_member

    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--train", type=int, default=16)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--test", type=int, default=3)
    ap.add_argument("--step", type=int, default=0, help="1: least-squares step of the correction")
    args = ap.parse_args(argv)
    members = lambda: (family_member(args.n, s) for s in range(1000, 1000 + args.train))
    prm, losses = train(members, args.epochs, args.lr)
    out = dict(n=args.n, train_systems=args.train, epochs=args.epochs, lr=args.lr,
               loss_first=float(np.mean(losses[:8])), loss_last=float(np.mean(losses[-8:])), systems=[])
    for s in range(900000, 900000 + args.test):
        out["systems"].append(dict(seed=s, **compare(prm, family_member(args.n, s), step=args.step)))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
