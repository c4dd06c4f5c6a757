"""ORACLE — test infrastructure, not product code.

CPU restatement of the learned preconditioner's network (senk_gb300/csrc/mpnn.cu)
in numpy float64: forward pass, loss and the hand-derived backward pass, with
the GPU's BF16 rounding points reproduced (``rounding=True``: GEMM operands, the
aggregated messages, the saved pre-activations) so that GPU gradients can be
checked against it; ``rounding=False`` gives the same network in plain float64,
whose backward pass the tests pin with finite differences.

There is no reference implementation of this part in SenK; the network is
defined by this file and the CUDA kernels together.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

HID, LAYERS, NIN = 64, 4, 3
OFF_WIN = 0
OFF_BIN = OFF_WIN + NIN * HID
OFF_LAYER = OFF_BIN + HID
LAYER_SIZE = 2 * HID * HID + HID
OFF_WOUT = OFF_LAYER + LAYERS * LAYER_SIZE
OFF_BOUT = OFF_WOUT + HID
NPARAMS = OFF_BOUT + 1


def bf16(x):
    """Round to bfloat16 (nearest, ties to even) through float32, as
    __float2bfloat16_rn does; returned as float64."""
    x32 = np.ascontiguousarray(np.asarray(x, np.float32))
    u = x32.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(P):
    P = np.asarray(P, np.float64)
    Win = P[OFF_WIN:OFF_BIN].reshape(NIN, HID)
    bin_ = P[OFF_BIN:OFF_LAYER]
    layers = []
    for l in range(LAYERS):
        o = OFF_LAYER + l * LAYER_SIZE
        layers.append((P[o:o + 2 * HID * HID].reshape(2 * HID, HID), P[o + 2 * HID * HID:o + LAYER_SIZE]))
    return Win, bin_, layers, P[OFF_WOUT:OFF_BOUT], P[OFF_BOUT]


def init_params(seed: int = 0) -> np.ndarray:
    """He-scaled random hidden weights, zero output layer (the network starts as
    plain ILU). float32."""
    rng = np.random.default_rng(seed)
    P = np.zeros(NPARAMS, np.float32)
    P[OFF_WIN:OFF_BIN] = rng.normal(0, np.sqrt(2.0 / NIN), NIN * HID)
    for l in range(LAYERS):
        o = OFF_LAYER + l * LAYER_SIZE
        # small residual branches keep the residual stream near its input scale
        P[o:o + 2 * HID * HID] = rng.normal(0, 0.5 * np.sqrt(2.0 / (2 * HID)), 2 * HID * HID)
    return P


class Graph:
    """Row-normalised |A| without the diagonal, and the node features of A."""

    def __init__(self, val, cind, rptr):
        N = len(rptr) - 1
        A = sp.csr_matrix((np.asarray(val, np.float64), np.asarray(cind), np.asarray(rptr)), shape=(N, N))
        diag = A.diagonal()
        absA = abs(A).tocsr()
        off = np.asarray(absA.sum(axis=1)).ravel() - np.abs(diag)
        Woff = absA - sp.diags(np.abs(diag))
        Woff.eliminate_zeros()
        inv = np.divide(1.0, off, out=np.zeros_like(off), where=off > 0)
        self.A = A
        self.A32 = sp.csr_matrix((A.data.astype(np.float32).astype(np.float64), A.indices, A.indptr), shape=A.shape)
        self.A32T = self.A32.T.tocsr()
        self.W = (sp.diags(inv) @ Woff).tocsr()
        # the GPU keeps W in FP32
        self.W.data = self.W.data.astype(np.float32).astype(np.float64)
        self.WT = self.W.T.tocsr()
        self.d = float(np.float32(diag.sum() / N))
        self.fd = (diag.astype(np.float32) / np.float32(self.d)).astype(np.float64)
        self.fs = ((off + np.abs(diag)).astype(np.float32) / np.float32(self.d)).astype(np.float64)
        self.n = N


def _round(x, on):
    return bf16(x) if on else np.asarray(x, np.float64)


def forward(P, g: Graph, r, rounding=True):
    """Returns (c, cache); c = net(r) per node."""
    Win, bin_, layers, wout, bout = unpack(P)
    r = np.asarray(r, np.float64)
    rms = np.sqrt(np.dot(r, r) / g.n)
    if rounding:
        inv = np.float64(np.float32(1.0 / rms))
        f2 = (r.astype(np.float32) * np.float32(inv)).astype(np.float64)
    else:
        inv = 1.0 / rms
        f2 = r * inv
    F = np.stack([g.fd, g.fs, f2], axis=1)
    z0 = F @ Win + bin_
    H = [np.maximum(z0, 0)]
    Xs, Zs = [], []
    for l in range(LAYERS):
        Th, beta = layers[l]
        xh = _round(H[l], rounding)
        m = _round(g.W @ xh, rounding)
        X = np.concatenate([xh, m], axis=1)
        z = X @ _round(Th, rounding) + beta
        Xs.append(X)
        Zs.append(_round(z, rounding))
        H.append(H[l] + np.maximum(z, 0))
    c = H[LAYERS] @ wout + bout
    return c, dict(F=F, z0=z0, H=H, X=Xs, Z=Zs, rms=rms, inv=inv)


def apply(P, g: Graph, r, ilu, rounding=True):
    """K(r) = ILU(r) + (rms / d) c."""
    c, cache = forward(P, g, r, rounding)
    return np.asarray(ilu, np.float64) + cache["rms"] / g.d * c


def apply_step(P, g: Graph, r, ilu, rounding=True):
    """K(r) = ILU(r) + alpha c with c = (rms / d) net(r) and
    alpha = (q . A c) / (A c . A c), q = r - A ILU(r): the alpha minimising
    |r - A K(r)| (senk_mpnn_set_step mode 1; 0 when A c = 0)."""
    c, cache = forward(P, g, r, rounding)
    ct = cache["rms"] / g.d * c
    ilu = np.asarray(ilu, np.float64)
    y = g.A @ ct
    q = np.asarray(r, np.float64) - g.A @ ilu
    den = float(y @ y)
    return ilu + (float(q @ y) / den if den > 0 else 0.0) * ct


def loss_grad(P, g: Graph, r, ilu, e, rounding=True, mode=1):
    """(loss, gradient) for one residual/error pair, as senk_mpnn_loss_grad.
    mode 1 (residual space): q = (r - A ILU(r)) / rms, loss = |A c / d - q|^2 / |q|^2;
    mode 0 (error space): t = (e - ILU(r)) d / rms, loss = |c - t|^2 / |t|^2."""
    Win, bin_, layers, wout, bout = unpack(P)
    c, ch = forward(P, g, r, rounding)
    if mode == 0:
        t = (np.asarray(e, np.float64) - np.asarray(ilu, np.float64)) * g.d * ch["inv"]
        if rounding:
            t = t.astype(np.float32).astype(np.float64)
        S = float(np.dot(t, t))
        diff = c - t
        loss = float(np.dot(diff, diff)) / S
        dc = 2.0 * diff / S
    else:
        q = (np.asarray(r, np.float64) - g.A @ np.asarray(ilu, np.float64)) * ch["inv"]
        if rounding:
            q = q.astype(np.float32).astype(np.float64)
        S = float(np.dot(q, q))
        res = g.A32 @ c / g.d - q
        loss = float(np.dot(res, res)) / S
        dc = 2.0 / (g.d * S) * (g.A32T @ res)
    G = np.zeros(NPARAMS)
    H = ch["H"]
    G[OFF_WOUT:OFF_BOUT] = H[LAYERS].T @ dc
    G[OFF_BOUT] = dc.sum()
    dH = np.outer(dc, wout)
    for l in range(LAYERS - 1, -1, -1):
        Th, _ = layers[l]
        gz = np.where(ch["Z"][l] > 0, dH, 0.0)
        o = OFF_LAYER + l * LAYER_SIZE
        G[o + 2 * HID * HID:o + LAYER_SIZE] = gz.sum(axis=0)
        dz = _round(gz, rounding)
        G[o:o + 2 * HID * HID] = (ch["X"][l].T @ dz).ravel()
        dX = dz @ _round(Th, rounding).T
        dH = dH + dX[:, :HID] + g.WT @ dX[:, HID:]
    g0 = np.where(ch["z0"] > 0, dH, 0.0)
    G[OFF_WIN:OFF_BIN] = (ch["F"].T @ g0).ravel()
    G[OFF_BIN:OFF_LAYER] = g0.sum(axis=0)
    return loss, G
