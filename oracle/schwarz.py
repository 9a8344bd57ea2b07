"""CPU restatement of the additive-Schwarz preconditioner (TEST INFRASTRUCTURE):
the aggregation, the coarse level's domains and the two-level application.

Restates crates/ppf-cts-solver/src/cpp/schwarz/schwarz.cu:551-645
(hem_partition): seeds visited in decreasing order of their summed coupling
to other vertices; each seed grows an aggregate to at most kmax members by
repeatedly absorbing the unassigned neighbour with the largest summed
coupling (float32 sums, in CSR order) to the aggregate; vertices left with no
positive coupling stay singletons. The reference orders seeds with an
unstable sort; this restatement, like the product, breaks ties by index.

Imported only by tests/ as the checker of ppf_schwarz_aggregate,
ppf_schwarz_coarsen and the PCG's Schwarz phases.
"""
from __future__ import annotations

import numpy as np

UNSET = 0xFFFFFFFF


def hem_aggregate(off, col, wgt, kmax: int):
    """(agg, n_agg) for the both-triangle CSR graph (off, col) with float32
    weights wgt."""
    off = np.asarray(off, np.int64)
    col = np.asarray(col, np.int64)
    wgt = np.asarray(wgt, np.float32)
    n = len(off) - 1
    incw = [0.0] * n
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            if col[k] != i:
                incw[i] += float(wgt[k])
    order = sorted(range(n), key=lambda i: -incw[i])
    agg = [UNSET] * n
    gain = [np.float32(0.0)] * n
    nid = 0
    for seed in order:
        if agg[seed] != UNSET:
            continue
        agg[seed] = nid
        size = 1
        touched = []

        def absorb(v):
            for k in range(off[v], off[v + 1]):
                u = int(col[k])
                if u == v or agg[u] != UNSET:
                    continue
                if gain[u] == 0.0:
                    touched.append(u)
                gain[u] = np.float32(gain[u] + wgt[k])

        absorb(seed)
        while size < kmax:
            best, bv = np.float32(0.0), UNSET
            for v in touched:
                if agg[v] == UNSET and gain[v] > best:
                    best, bv = gain[v], v
            if bv == UNSET:
                break
            agg[bv] = nid
            size += 1
            absorb(bv)
        for v in touched:
            gain[v] = np.float32(0.0)
        nid += 1
    return np.array(agg, np.uint32), nid


def galerkin_domains(off, col, blocks, agg, n_agg: int, kmax: int):
    """(dom, n_dom): the coarse level's domains.

    Restates the two-level construction of
    crates/ppf-cts-solver/src/cpp/schwarz/schwarz.cu:1225-1327 (Galerkin
    blocks C A C^T of the aggregates) and 1416-1470 (grouping the coarse
    nodes into domains of at most kmax), with the grouping done by the
    heavy-edge growth above on the Frobenius norms of the Galerkin blocks.
    The blocks of distinct aggregate pairs are summed in float32 over the rows
    in order and each row's entries in order; `blocks` holds the 9 values of
    every CSR entry (column-major)."""
    off = np.asarray(off, np.int64)
    col = np.asarray(col, np.int64)
    blocks = np.asarray(blocks, np.float32).reshape(-1, 9)
    agg = np.asarray(agg, np.int64)
    n = len(off) - 1
    rows = [dict() for _ in range(n_agg)]
    for i in range(n):
        g = int(agg[i])
        for k in range(off[i], off[i + 1]):
            h = int(agg[col[k]])
            if h == g:
                continue
            acc = rows[g].get(h)
            if acc is None:
                acc = rows[g][h] = np.zeros(9, np.float32)
            acc += blocks[k]  # elementwise float32 additions
    coff, ccol, cw = [0], [], []
    for g in range(n_agg):
        for h in sorted(rows[g]):
            s = rows[g][h]
            w = np.float32(0.0)
            for q in range(9):
                w = np.float32(w + np.float32(s[q] * s[q]))
            ccol.append(h)
            cw.append(np.float32(np.sqrt(w)))
        coff.append(len(ccol))
    return hem_aggregate(coff, ccol, np.array(cw, np.float32), kmax)


def _dense_inverse_apply(M, v):
    """(M + floor I)^{-1} v for one dense block, with the diagonal floor of
    schwarz.cu:234-246 (1e-6 of the mean diagonal plus 1e-8)."""
    d = len(M)
    fl = 1e-6 * np.trace(M) / d + 1e-8
    L = np.linalg.cholesky(M + fl * np.eye(d))
    y = np.linalg.solve(L, v)
    return np.linalg.solve(L.T, y)


def schwarz_apply(A, agg, r, dom=None, weight: float = 1.0):
    """z = S_0 r (+ w C^T S_1 C r with dom) in float64 for the both-triangle
    operator A (scipy sparse, 3n x 3n): S_0 the per-aggregate inverse of the
    floored dense block (members in ascending order), C the piecewise-constant
    restriction onto aggregates, S_1 the per-domain inverse of the floored
    Galerkin block (schwarz.cu:315-374 and 1560-1600)."""
    import scipy.sparse as sp

    agg = np.asarray(agg, np.int64)
    r = np.asarray(r, np.float64).reshape(-1)
    n = len(agg)
    n_agg = int(agg.max()) + 1
    z = np.zeros(3 * n)
    A = sp.csr_matrix(A)
    for g in range(n_agg):
        mem = np.flatnonzero(agg == g)
        idx = (3 * mem[:, None] + np.arange(3)).reshape(-1)
        z[idx] = _dense_inverse_apply(A[idx][:, idx].toarray(), r[idx])
    if dom is None:
        return z
    dom = np.asarray(dom, np.int64)
    C = sp.csr_matrix((np.ones(3 * n), ((3 * agg[:, None] + np.arange(3)).reshape(-1),
                                        np.arange(3 * n))), shape=(3 * n_agg, 3 * n))
    Ac = (C @ A @ C.T).tocsr()
    rc = C @ r
    ec = np.zeros(3 * n_agg)
    for D in range(int(dom.max()) + 1):
        mem = np.flatnonzero(dom == D)
        idx = (3 * mem[:, None] + np.arange(3)).reshape(-1)
        ec[idx] = _dense_inverse_apply(Ac[idx][:, idx].toarray(), rc[idx])
    return z + weight * (C.T @ ec)
