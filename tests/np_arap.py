"""Independent numpy/scipy FP64 restatement of inc/deform/arap.h (test-only).

It shares no code with the C oracle: cotan weights are vectorised over faces
(arap.h:182-239), rotations come from LAPACK's SVD via ``np.linalg.svd``
(arap.h:376-382) and the global step uses SuperLU (``scipy.sparse.linalg.splu``)
instead of an LDL^T (arap.h:337,420). Agreement of the two restatements to
~1e-12 guards the C oracle, which the CUDA library is checked against.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def cotan_weights(pos: np.ndarray, faces: np.ndarray) -> sp.csr_matrix:
    """arap.h:182-239: clamped Heron cotangents, 1/2 per face, both directions."""
    v0, v1, v2 = pos[faces[:, 0]], pos[faces[:, 1]], pos[faces[:, 2]]
    l0 = np.sqrt(np.maximum(1e-8, ((v1 - v0) ** 2).sum(1)))
    l1 = np.sqrt(np.maximum(1e-8, ((v2 - v1) ** 2).sum(1)))
    l2 = np.sqrt(np.maximum(1e-8, ((v0 - v2) ** 2).sum(1)))
    s = 0.5 * (l0 + l1 + l2)
    with np.errstate(invalid="ignore"):
        area = np.sqrt(s * (s - l0) * (s - l1) * (s - l2))
    area = np.where(np.isnan(area), 1e-8, np.maximum(1e-8, area))
    denom = 1.0 / (4.0 * area)
    cots = [(-l0 * l0 + l1 * l1 + l2 * l2) * denom,
            (l0 * l0 - l1 * l1 + l2 * l2) * denom,
            (l0 * l0 + l1 * l1 - l2 * l2) * denom]
    cots = [np.maximum(1e-10, c) * 0.5 for c in cots]
    edges = [(faces[:, 0], faces[:, 1]), (faces[:, 1], faces[:, 2]), (faces[:, 2], faces[:, 0])]
    rows, cols, vals = [], [], []
    for (a, b), c in zip(edges, cots):
        rows += [a, b]
        cols += [b, a]
        vals += [c, c]
    V = len(pos)
    W = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(V, V))
    return W.tocsr()


def rotations(W: sp.csr_matrix, p: np.ndarray, pp: np.ndarray) -> np.ndarray:
    """arap.h:354-384 with LAPACK's SVD."""
    V = len(p)
    Wc = W.tocoo()
    e = p[Wc.row] - p[Wc.col]
    f = pp[Wc.row] - pp[Wc.col]
    outer = Wc.data[:, None, None] * e[:, :, None] * f[:, None, :]
    cov = np.zeros((V, 3, 3))
    np.add.at(cov, Wc.row, outer)
    U, S, Vt = np.linalg.svd(cov)
    Vm = np.swapaxes(Vt, 1, 2)
    Ut = np.swapaxes(U, 1, 2)
    d = np.linalg.det(Vm @ Ut)
    D = np.zeros((V, 3, 3))
    D[:, 0, 0] = 1.0
    D[:, 1, 1] = 1.0
    D[:, 2, 2] = d
    return Vm @ D @ Ut


def deform(pos: np.ndarray, faces: np.ndarray, cidx, ctargets, iterations: int):
    """A dirty deform(iterations) from rest = pos. Returns (ok, positions)."""
    V = len(pos)
    p = pos.astype(np.float64).copy()
    W = cotan_weights(p, faces)
    cidx = np.asarray(cidx, np.int64)
    constrained = np.zeros(V, bool)
    constrained[cidx] = True
    pp = p.copy()
    pp[cidx] = ctargets
    free = np.nonzero(~constrained)[0]
    m = len(free)
    if m == V:
        return True, pos.copy()
    fidx = -np.ones(V, np.int64)
    fidx[free] = np.arange(m)
    Wc = W.tocoo()
    diag = np.asarray(W.sum(1)).ravel()
    keep = (~constrained[Wc.row]) & (~constrained[Wc.col])
    L = sp.coo_matrix((-Wc.data[keep], (fidx[Wc.row[keep]], fidx[Wc.col[keep]])), shape=(m, m)).tocsc()
    L = L + sp.diags(diag[free])
    cm = (~constrained[Wc.row]) & constrained[Wc.col]
    bfixed = np.zeros((m, 3))
    np.add.at(bfixed, fidx[Wc.row[cm]], Wc.data[cm, None] * pp[Wc.col[cm]])
    lu = spla.splu(L.tocsc())
    rowsf = ~constrained[Wc.row]
    for _ in range(iterations):
        R = rotations(W, p, pp)
        r = R[Wc.row] + R[Wc.col]
        d = p[Wc.row] - p[Wc.col]
        pt = np.einsum("eij,ej->ei", r, d) * (Wc.data * 0.5)[:, None]
        b = bfixed.copy()
        np.add.at(b, fidx[Wc.row[rowsf]], pt[rowsf])
        x = lu.solve(b)
        pp[free] = x
    return True, pp
