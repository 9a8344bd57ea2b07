"""CPU oracle of the FSAI factor -- test infrastructure only.

Restates, in numpy (float64 solves on the float32 system), the block
factorised sparse approximate inverse that csrc/gpu/fsai.cu builds
(Kolotilina and Yeremin's FSAI in 3x3 blocks of the block-Jacobi-normalised
operator Â = C^{-1} A C^{-T}). The reference has no such preconditioner: its
PCG uses block-Jacobi (crates/ppf-cts-solver/src/cpp/solver/solver.cu:357-400).

For vertex i with kept lower neighbours J (fixed transpose list, then the
contact one, Dirichlet vertices left out; at most 15, the strongest by
|Â(i, j)|_F when there are more, ties to the earlier one) and P = (J, i):
    Y = Â[P, P]^{-1} E_i,  Y(i) = L L^T,  Ĝ(i, P) = L^{-1} Y^T
and G = Ĝ C^{-1}.
"""
from __future__ import annotations

import numpy as np

from . import learned as OL

MAX_LOWER = 15


def _blocks(g: OL.Graph):
    """(row, col) -> upper block [3, 3] of both parts (row < col, or diagonal)."""
    out = {}
    for p in range(2):
        off, col, blk, row = g.parts[p]
        for k in range(len(col)):
            out[(int(row[k]), int(col[k]))] = blk[k]
    return out


def kept_neighbours(g: OL.Graph, i: int):
    """The kept lower neighbours of vertex i as (vertex, edge index) pairs, in
    candidate order."""
    cands = []
    for p in range(2):
        tr_off, tr = g.tr[p]
        base = 0 if p == 0 else g.nnz_f
        for t in range(int(tr_off[i]), int(tr_off[i + 1])):
            r, k = int(tr[t, 0]), int(tr[t, 1])
            cands.append((r, base + k))
    norms = np.array([-1.0 if g.dof[r] else float(OL._fro(g.ah[e:e + 1])[0]) for r, e in cands],
                     np.float32)
    live = [t for t in range(len(cands)) if norms[t] >= 0]
    if len(live) <= MAX_LOWER:
        return [cands[t] for t in live]
    order = sorted(live, key=lambda t: (-float(norms[t]), t))[:MAX_LOWER]
    return [cands[t] for t in sorted(order)]


def factor(g: OL.Graph):
    """(gdiag [n, 3, 3], gedge {edge index: G(hi, lo) [3, 3]}, kept {i: [...]})
    in float64; rows of Dirichlet vertices keep G(i, i) = C(i)^{-1}."""
    blocks = _blocks(g)
    cinv = g.cinv.astype(np.float64)
    gdiag = np.zeros((g.n, 3, 3))
    gedge = {}
    kept = {}
    for i in range(g.n):
        if g.dof[i]:
            gdiag[i] = cinv[i]
            continue
        J = kept_neighbours(g, i)
        kept[i] = J
        P = [v for v, _ in J] + [i]
        m = len(J)
        M = np.zeros((3 * (m + 1), 3 * (m + 1)))
        for a, va in enumerate(P):
            for b, vb in enumerate(P):
                if a == b:
                    blk = cinv[va] @ g.A_ii[va].astype(np.float64) @ cinv[va].T
                elif b == m:
                    blk = g.ah[J[a][1]].astype(np.float64).T
                elif a == m:
                    blk = g.ah[J[b][1]].astype(np.float64)
                else:
                    lo, hi = min(va, vb), max(va, vb)
                    U = blocks.get((lo, hi))
                    U = np.zeros((3, 3)) if U is None else U.astype(np.float64)
                    Aab = U if va < vb else U.T
                    blk = cinv[va] @ Aab @ cinv[vb].T
                M[3 * a:3 * a + 3, 3 * b:3 * b + 3] = blk
        E = np.zeros((3 * (m + 1), 3))
        E[3 * m:, :] = np.eye(3)
        Y = np.linalg.solve(0.5 * (M + M.T), E)
        Yii = 0.5 * (Y[3 * m:] + Y[3 * m:].T)
        L3inv = np.linalg.inv(np.linalg.cholesky(Yii))
        Ghat = L3inv @ Y.T  # [3, 3 (m + 1)]
        for a, (v, e) in enumerate(J):
            gedge[e] = Ghat[:, 3 * a:3 * a + 3] @ cinv[v]
        gdiag[i] = Ghat[:, 3 * m:] @ cinv[i]
    return gdiag, gedge, kept


def dense_factor(g: OL.Graph, gdiag, gedge):
    """G as a dense (3n x 3n) matrix (small cases)."""
    G = np.zeros((3 * g.n, 3 * g.n))
    for i in range(g.n):
        G[3 * i:3 * i + 3, 3 * i:3 * i + 3] = gdiag[i]
    for e, blk in gedge.items():
        hi, lo = int(g.hi[e]), int(g.lo[e])
        G[3 * hi:3 * hi + 3, 3 * lo:3 * lo + 3] = blk
    return G


def dense_operator(g: OL.Graph):
    """A on the free vertices (Dirichlet rows and columns as identity) as a
    dense (3n x 3n) matrix."""
    A = np.zeros((3 * g.n, 3 * g.n))
    blocks = _blocks(g)
    for (r, c), blk in blocks.items():
        if g.dof[r] or g.dof[c]:
            continue
        b = blk.astype(np.float64)
        A[3 * r:3 * r + 3, 3 * c:3 * c + 3] = b
        if r != c:
            A[3 * c:3 * c + 3, 3 * r:3 * r + 3] = b.T
    for i in range(g.n):
        if g.dof[i]:
            A[3 * i:3 * i + 3, 3 * i:3 * i + 3] = np.eye(3)
    return A
