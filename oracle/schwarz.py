"""CPU restatement of the additive-Schwarz aggregation (TEST INFRASTRUCTURE).

Restates crates/ppf-cts-solver/src/cpp/schwarz/schwarz.cu:551-645
(hem_partition): seeds visited in decreasing order of their summed coupling
to other vertices; each seed grows an aggregate to at most kmax members by
repeatedly absorbing the unassigned neighbour with the largest summed
coupling (float32 sums, in CSR order) to the aggregate; vertices left with no
positive coupling stay singletons. The reference orders seeds with an
unstable sort; this restatement, like the product, breaks ties by index.

Imported only by tests/ as the checker of ppf_schwarz_aggregate.
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
