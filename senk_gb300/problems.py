"""Seeded synthetic problems of the shapes the solver path is measured on.

The reference's drivers read SuiteSparse MatrixMarket files (main.cpp:11-25), which
are not available; these generators stand in for them.  Every generator returns a
CSR matrix with sorted column indices and a diagonal entry in every row (the
contract of senk::matrix::CheckStructure, include/senk_matrix.hpp:45-56), as
numpy arrays ``(val float64, cind int32, rptr int32)``.

Workloads:
  * ``poisson2d(128)``        2D 5-point Poisson, N=16,384, nnz=81,408; b = A*1.
  * ``convdiff3d(128, 0.5)``  3D 7-point upwind convection-diffusion, N=2,097,152,
    nnz=14,581,760; unit diffusion, velocity (1,1,1), cell Peclet Pe = v*h/(2D):
    scaled stencil diagonal 6+6Pe, upwind neighbour -(1+2Pe), downwind -1.
  * ``vardiff3d(160, ...)``   3D 7-point diffusion with face coefficients
    exp((g_p+g_q)/2) of a Gaussian random field g (FFT spectral synthesis,
    Gaussian covariance with correlation length ``corr`` cells, std ``sigma``);
    boundary faces use the cell's own exp(g_p) (zero Dirichlet ghost).
  * ``block27(96, ...)``      block-3x3 system on an n^3 grid with a 27-point
    stencil: dense 3x3 off-diagonal blocks with entries U(-1, 0) * scale, SPD
    diagonal blocks S S^T + c I with c chosen so that the smallest eigenvalue of
    each diagonal block is at least 1.1 times the sum of the spectral norms of
    its row's off-diagonal blocks (block diagonal dominance 1.1). N = 3 n^3 rows,
    nnz = 9 * (number of nonzero blocks), as generated (no "71M" rounding).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Csr:
    """A CSR matrix in the reference's layout: val[nnz], cind[nnz], rptr[N+1]."""

    val: np.ndarray
    cind: np.ndarray
    rptr: np.ndarray

    @property
    def n(self) -> int:
        return int(self.rptr.shape[0] - 1)

    @property
    def nnz(self) -> int:
        return int(self.rptr[-1])

    def copy(self) -> "Csr":
        return Csr(self.val.copy(), self.cind.copy(), self.rptr.copy())

    def astype(self, dtype) -> "Csr":
        return Csr(self.val.astype(dtype), self.cind, self.rptr)

    def matvec(self, x: np.ndarray) -> np.ndarray:
        """y = A x in float64 (row sums in index order), for building right-hand sides."""
        rows = np.repeat(np.arange(self.n), np.diff(self.rptr))
        prod = self.val.astype(np.float64) * x[self.cind]
        return np.bincount(rows, weights=prod, minlength=self.n)


def _assemble(cols: np.ndarray, vals: np.ndarray, mask: np.ndarray) -> Csr:
    """Rows are the first axis; entries per row are already in column order."""
    counts = mask.sum(axis=1).astype(np.int64)
    rptr = np.zeros(cols.shape[0] + 1, dtype=np.int64)
    np.cumsum(counts, out=rptr[1:])
    return Csr(np.ascontiguousarray(vals[mask], dtype=np.float64),
               np.ascontiguousarray(cols[mask], dtype=np.int32),
               rptr.astype(np.int32))


def poisson2d(n: int = 128) -> Csr:
    """5-point Laplacian on an n x n grid, row r = j*n + i, Dirichlet boundary."""
    N = n * n
    r = np.arange(N, dtype=np.int64)
    i, j = r % n, r // n
    offs = [-n, -1, 0, 1, n]
    ok = [j > 0, i > 0, np.ones(N, bool), i < n - 1, j < n - 1]
    cols = np.stack([r + o for o in offs], axis=1)
    vals = np.stack([np.full(N, 4.0 if o == 0 else -1.0) for o in offs], axis=1)
    return _assemble(cols, vals, np.stack(ok, axis=1))


def convdiff3d(n: int = 128, pe: float = 0.5) -> Csr:
    """7-point upwind convection-diffusion, v=(1,1,1), cell Peclet ``pe``."""
    N = n ** 3
    r = np.arange(N, dtype=np.int64)
    i, j, k = r % n, (r // n) % n, r // (n * n)
    n2 = n * n
    up, down, diag = -(1.0 + 2.0 * pe), -1.0, 6.0 + 6.0 * pe
    offs = [(-n2, k > 0, up), (-n, j > 0, up), (-1, i > 0, up), (0, None, diag),
            (1, i < n - 1, down), (n, j < n - 1, down), (n2, k < n - 1, down)]
    cols = np.stack([r + o for o, _, _ in offs], axis=1)
    vals = np.stack([np.full(N, v) for _, _, v in offs], axis=1)
    mask = np.stack([np.ones(N, bool) if m is None else m for _, m, _ in offs], axis=1)
    return _assemble(cols, vals, mask)


def gaussian_random_field(n: int, sigma: float, corr: float, seed: int) -> np.ndarray:
    """Zero-mean field on an n^3 grid with Gaussian covariance exp(-d^2/(2 corr^2)).

    White noise from ``numpy.random.default_rng(seed)`` is filtered in Fourier
    space by the square root of the covariance's spectrum, exp(-(corr*|k|)^2/4),
    then standardised to standard deviation ``sigma``.  Array index order is
    [k][j][i] (i fastest), matching the row numbering of the matrices.
    """
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((n, n, n))
    kf = 2.0 * np.pi * np.fft.fftfreq(n)
    kr = 2.0 * np.pi * np.fft.rfftfreq(n)
    k2 = kf[:, None, None] ** 2 + kf[None, :, None] ** 2 + kr[None, None, :] ** 2
    g = np.fft.irfftn(np.fft.rfftn(w) * np.exp(-(corr ** 2) * k2 / 4.0), s=(n, n, n), axes=(0, 1, 2))
    g -= g.mean()
    g *= sigma / g.std()
    return g


def vardiff3d(n: int = 160, sigma: float = 1.5, corr: float = 8.0, seed: int = 0) -> Csr:
    """7-point variable-coefficient diffusion with log-normal coefficients."""
    g = gaussian_random_field(n, sigma, corr, seed).reshape(-1)
    N = n ** 3
    r = np.arange(N, dtype=np.int64)
    i, j, k = r % n, (r // n) % n, r // (n * n)
    n2 = n * n
    kap = np.exp(g)
    faces = [(-n2, k > 0), (-n, j > 0), (-1, i > 0), (1, i < n - 1), (n, j < n - 1), (n2, k < n - 1)]
    off_vals = []
    diag = np.zeros(N)
    for o, ok in faces:
        nb = np.where(ok, r + o, r)
        kf = np.where(ok, np.exp(0.5 * (g + g[nb])), kap)
        diag += kf
        off_vals.append(-kf)
    cols = np.stack([r + o for o, _ in faces[:3]] + [r] + [r + o for o, _ in faces[3:]], axis=1)
    vals = np.stack(off_vals[:3] + [diag] + off_vals[3:], axis=1)
    mask = np.stack([ok for _, ok in faces[:3]] + [np.ones(N, bool)] + [ok for _, ok in faces[3:]], axis=1)
    return _assemble(cols, vals, mask)


def uniform_solution(n: int, seed: int = 0) -> np.ndarray:
    """x_true ~ U(-1, 1) from numpy.random.default_rng(seed)."""
    return np.random.default_rng(seed).uniform(-1.0, 1.0, n)


def normal_solution(n: int, seed: int = 1) -> np.ndarray:
    """x_true ~ N(0, 1) from numpy.random.default_rng(seed)."""
    return np.random.default_rng(seed).standard_normal(n)


def _sym3_max_eig(M: np.ndarray) -> np.ndarray:
    """Largest eigenvalue of each symmetric 3x3 matrix in M[..., 3, 3], by the
    closed-form trigonometric solution of the characteristic cubic (Smith,
    "Eigenvalues of a symmetric 3 x 3 matrix", CACM 4(4), 1961)."""
    q = (M[..., 0, 0] + M[..., 1, 1] + M[..., 2, 2]) / 3.0
    p1 = M[..., 0, 1] ** 2 + M[..., 0, 2] ** 2 + M[..., 1, 2] ** 2
    p2 = (M[..., 0, 0] - q) ** 2 + (M[..., 1, 1] - q) ** 2 + (M[..., 2, 2] - q) ** 2 + 2.0 * p1
    p = np.sqrt(p2 / 6.0)
    safe = np.where(p > 0, p, 1.0)
    b00, b11, b22 = (M[..., 0, 0] - q) / safe, (M[..., 1, 1] - q) / safe, (M[..., 2, 2] - q) / safe
    b01, b02, b12 = M[..., 0, 1] / safe, M[..., 0, 2] / safe, M[..., 1, 2] / safe
    det = b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02)
    phi = np.arccos(np.clip(det / 2.0, -1.0, 1.0)) / 3.0
    return np.where(p > 0, q + 2.0 * p * np.cos(phi), q)


def block27(n: int = 96, scale: float = 1.0, dominance: float = 1.1, seed: int = 0) -> Csr:
    """Block-3x3 system on an n^3 grid with a 27-point stencil (3 unknowns per
    node, node-major: row 3*node + k), seeded. Off-diagonal blocks: entries
    U(-1, 0) * scale; diagonal blocks S S^T + c I with S ~ U(-1, 1) and c chosen
    so that their smallest eigenvalue is at least `dominance` times the sum of
    the spectral norms of the row's off-diagonal blocks (plus 1e-3)."""
    rng = np.random.default_rng([seed, 27])
    nn = n ** 3
    node = np.arange(nn, dtype=np.int64)
    i, j, k = node % n, (node // n) % n, node // (n * n)
    nbrs, keep = [], []
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                ii, jj, kk = i + di, j + dj, k + dk
                ok = (ii >= 0) & (ii < n) & (jj >= 0) & (jj < n) & (kk >= 0) & (kk < n)
                nbrs.append(ii + n * jj + n * n * kk)
                keep.append(ok)
    nbrs = np.stack(nbrs, axis=1)        # nn x 27, ascending node index (dk, dj, di order)
    keep = np.stack(keep, axis=1)
    blocks = rng.uniform(0.0, 1.0, (nn, 27, 3, 3))
    np.multiply(blocks, -scale, out=blocks)
    blocks[~keep] = 0.0
    centre = 13                           # (0, 0, 0)
    # spectral norms of the off-diagonal blocks: sqrt of the largest eigenvalue of B^T B
    offsum = np.zeros(nn)
    for t in range(27):
        if t == centre:
            continue
        B = blocks[:, t]
        offsum += np.sqrt(np.maximum(_sym3_max_eig(np.einsum("nki,nkj->nij", B, B)), 0.0))
    S = rng.uniform(-1.0, 1.0, (nn, 3, 3))
    D = S @ np.transpose(S, (0, 2, 1))
    lam = np.linalg.eigvalsh(D)[:, 0]
    c = np.maximum(dominance * offsum - lam, 0.0) + 1e-3
    blocks[:, centre] = D + c[:, None, None] * np.eye(3)
    # scalar CSR: row 3*node + a, columns 3*nbr + b for each kept neighbour
    cnt = keep.sum(axis=1) * 3
    rptr = np.zeros(3 * nn + 1, np.int64)
    rptr[1:] = np.cumsum(np.repeat(cnt, 3))
    vals = np.ascontiguousarray(np.transpose(blocks, (0, 2, 1, 3)))    # node, a, nbr, b
    del blocks
    mask = np.broadcast_to(keep[:, None, :, None], (nn, 3, 27, 3))
    val = vals[mask]
    del vals
    cols = (3 * nbrs[:, :, None] + np.arange(3)[None, None, :]).astype(np.int32)   # nn x 27 x 3
    col = np.broadcast_to(cols[:, None, :, :], (nn, 3, 27, 3))[mask]
    return Csr(np.ascontiguousarray(val, np.float64), np.ascontiguousarray(col, np.int32), rptr.astype(np.int32))


def block27_node_graph(n: int) -> Csr:
    """Node graph of block27(n) (one entry per nonzero block), from the stencil."""
    nn = n ** 3
    node = np.arange(nn, dtype=np.int64)
    i, j, k = node % n, (node // n) % n, node // (n * n)
    nbrs, keep = [], []
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                ii, jj, kk = i + di, j + dj, k + dk
                nbrs.append(ii + n * jj + n * n * kk)
                keep.append((ii >= 0) & (ii < n) & (jj >= 0) & (jj < n) & (kk >= 0) & (kk < n))
    nbrs, keep = np.stack(nbrs, axis=1), np.stack(keep, axis=1)
    rptr = np.zeros(nn + 1, np.int64)
    rptr[1:] = np.cumsum(keep.sum(axis=1))
    return Csr(np.ones(int(rptr[-1])), nbrs[keep].astype(np.int32), rptr.astype(np.int32))


def expand_node_permutation(LP_nodes: np.ndarray, bs: int = 3) -> tuple:
    """Scalar-row permutations (LP, RP) of a node permutation, bs rows per node:
    new scalar row bs*i + a is old row bs*LP_nodes[i] + a."""
    LP = (bs * np.asarray(LP_nodes, np.int64)[:, None] + np.arange(bs)[None, :]).reshape(-1)
    RP = np.empty_like(LP)
    RP[LP] = np.arange(LP.size)
    return LP.astype(np.int32), RP.astype(np.int32)


def node_graph(A: Csr, bs: int = 3) -> Csr:
    """Pattern of the node graph of a block matrix (one entry per nonzero block)."""
    nrows = A.n // bs
    rows = np.repeat(np.arange(A.n), np.diff(A.rptr)) // bs
    cols = A.cind.astype(np.int64) // bs
    key = np.unique(rows * nrows + cols)
    r, c = key // nrows, key % nrows
    rptr = np.zeros(nrows + 1, np.int64)
    np.add.at(rptr, r + 1, 1)
    return Csr(np.ones(key.size), c.astype(np.int32), np.cumsum(rptr).astype(np.int32))
