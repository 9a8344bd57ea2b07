"""Small Newton-system-shaped graphs for the learned preconditioner's tests.

synthetic(): a random SPD block system with a fixed pattern (a chain plus
random couplings, diagonal blocks included), contact blocks outside it and
two Dirichlet vertices, in the layout the solver dumps (upper CSR, 9
column-major floats per block). Small enough for the oracle's loops.
"""
import numpy as np


def _csr(n, pairs):
    rows = [[] for _ in range(n)]
    for i, j in pairs:
        rows[min(i, j)].append(max(i, j))
    off = [0]
    col = []
    for i in range(n):
        r = sorted(set(rows[i]))
        col += r
        off.append(len(col))
    return np.array(off, np.uint32), np.array(col, np.uint32)


def synthetic(n=40, seed=0, dirichlet=(3, 17), hub=0):
    """hub > 0: the last vertex also gets contact couplings to the first `hub`
    vertices (a row with more lower neighbours than a factor keeps)."""
    rng = np.random.default_rng(seed)
    fixed = [(i, i) for i in range(n)] + [(i, i + 1) for i in range(n - 1)]
    fixed += [(int(a), int(b)) for a, b in rng.integers(0, n, (n, 2)) if a != b]
    f_off, f_col = _csr(n, fixed)
    fset = {(min(a, b), max(a, b)) for a, b in fixed}
    contact = [(int(a), int(b)) for a, b in rng.integers(0, n, (n // 2, 2))
               if a != b and (min(a, b), max(a, b)) not in fset]
    contact += [(j, n - 1) for j in range(hub) if (j, n - 1) not in fset]
    c_off, c_col = _csr(n, contact)
    dof = np.zeros(n, np.uint32)
    dof[list(dirichlet)] = 1

    def blocks(off, col):
        vals = np.zeros((len(col), 3, 3), np.float32)
        row = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
        for k in range(len(col)):
            if row[k] == col[k]:
                continue
            m = rng.normal(0, 0.3, (3, 3))
            vals[k] = (0.5 * (m + m.T) if rng.random() < 0.5 else m).astype(np.float32)
            if dof[row[k]] or dof[col[k]]:
                vals[k] = 0  # eliminated
        return row, vals

    f_row, f_blk = blocks(f_off, f_col)
    c_row, c_blk = blocks(c_off, c_col)
    # diagonal blocks: SPD, dominant over each row's couplings
    load = np.zeros(n)
    for row, col, blk in ((f_row, f_col, f_blk), (c_row, c_col, c_blk)):
        for k in range(len(col)):
            s = np.abs(blk[k]).sum()
            load[row[k]] += s
            load[col[k]] += s
    for k in np.nonzero(f_row == f_col)[0]:
        i = f_row[k]
        m = rng.normal(0, 0.2, (3, 3))
        f_blk[k] = (m @ m.T + (0.6 * load[i] + 1.0) * np.eye(3)).astype(np.float32)
        if dof[i]:
            f_blk[k] = np.eye(3, dtype=np.float32)
    colmajor = lambda b: np.ascontiguousarray(b.transpose(0, 2, 1).reshape(-1), np.float32)
    mass = rng.uniform(0.5, 2.0, n).astype(np.float32)
    return {
        "n": n, "f_off": f_off, "f_col": f_col, "f_val": colmajor(f_blk),
        "d_off": c_off, "d_col": c_col, "d_val": colmajor(c_blk),
        "dof": dof, "mass": mass,
    }


def graph(s):
    from oracle import learned as L

    return L.Graph(int(s["n"]), (s["f_off"], s["f_col"], s["f_val"]),
                   (s["d_off"], s["d_col"], s["d_val"]), s["dof"], s["mass"])


def probes(n, W=4, seed=0):
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 2, (W, n, 3)) * 2 - 1).astype(np.float32)
