"""CPU oracle of the learned PCG preconditioner -- test infrastructure only.

The reference has no learned preconditioner: its PCG uses block-Jacobi
(crates/ppf-cts-solver/src/cpp/solver/solver.cu:357-400). This module restates,
in numpy, the network that the sm_103a kernels of csrc/gpu/learned.cu evaluate
and train, so the tests can check the kernels' outputs and gradients against
it; nothing in the product imports it.

The network reads one Newton system A (the operator the PCG solves: fixed
pattern plus contact blocks, after Dirichlet elimination) and emits the factor
of the preconditioner P = G^T G + eps D^{-1}, G = Ĝ C^{-1}, on A's own pattern:

    Ĝ(i, i)   = d_i I,                d_i = exp(clamp(q_i, -4, 4))
    Ĝ(hi, lo) = -alpha_e Â(hi, lo),   alpha_e = 2 sigmoid(o_e)

where Â = C^{-1} A C^{-T} (C: lower Cholesky factor of each diagonal block).
Weights are bf16, activations are rounded to bf16 where they feed a matrix
product, products accumulate in fp32.

Layers (hidden width 32; every layer input carries a constant-1 column that
holds the bias):
    X0  = [node features (15), 1]                          n x 16
    H0  = bf16(relu(X0 W0^T))                              n x 32
    Xl  = [H(l-1), bf16(mean over neighbours of H(l-1)), 1, 0...]  n x 80
    Hl  = bf16(relu(Xl Wl^T)),  l = 1, 2, 3
    Xh  = [H3, 1, 0...]                                    n x 48
    Y   = Xh Wh^T  (fp32)                                  n x 80
    per edge (hi > lo):  f = bf16([Â(hi, lo) (9, column-major), |Â(hi, lo)|_F, 1, 0...])
        z = relu(Y[hi, 0:32] + Y[lo, 32:64] + Wf f),  o = wo . [z, 1]
    q_i = Y[i, 64]

Training minimises Kaporin's condition number of M = Ĝ Â Ĝ^T, whose minimiser
over a fixed pattern is the factorised sparse approximate inverse:
    L = ln(tr(M) / N) - (1/N) ln det(Ĝ)^2   (+ the constant ln det(Â) / N)
with N = 3 n_free, tr(M) estimated by W Rademacher probes w: tr M ~ (1/W)
sum_w (Ĝ^T w)^T Â (Ĝ^T w), and ln det Ĝ^2 = 6 sum_i ln d_i.
"""
from __future__ import annotations

import numpy as np

H = 32
OFF_W0, OFF_W1, OFF_WH, OFF_WF, OFF_WO = 0, 512, 8192, 12032, 12544
N_WEIGHTS = 12592
IN0, INL, INH, OUTH, INF = 16, 80, 48, 80, 16
CLAMP_Q = 4.0


def weight_views(w):
    """Named views of a flat weight blob (row-major [out][in] matrices)."""
    w = np.asarray(w)
    return {
        "W0": w[OFF_W0:OFF_W0 + 32 * IN0].reshape(32, IN0),
        "W1": w[OFF_W1:OFF_W1 + 32 * INL].reshape(32, INL),
        "W2": w[OFF_W1 + 32 * INL:OFF_W1 + 64 * INL].reshape(32, INL),
        "W3": w[OFF_W1 + 64 * INL:OFF_W1 + 96 * INL].reshape(32, INL),
        "Wh": w[OFF_WH:OFF_WH + OUTH * INH].reshape(OUTH, INH),
        "Wf": w[OFF_WF:OFF_WF + 32 * INF].reshape(32, INF),
        "wo": w[OFF_WO:OFF_WO + 48],
    }


_EXACT = [False]


class exact_arithmetic:
    """Within this context bf16() rounds nothing, so the loss is a smooth
    function of the weights and the gradient can be checked by finite
    differences."""

    def __enter__(self):
        _EXACT[0] = True

    def __exit__(self, *a):
        _EXACT[0] = False


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), kept as float32."""
    x = np.ascontiguousarray(x, np.float32)
    if _EXACT[0]:
        return x.copy()
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(x), x, out).reshape(x.shape)


def bf16_bits(x):
    """float32 -> bfloat16 bit patterns (uint16)."""
    return (bf16(x).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, np.uint32) << 16).view(np.float32)


# ---- the system as a graph ----------------------------------------------------------


def _cols(blocks):
    """9 column-major floats per block -> [k, 3, 3] with [k, r, c]."""
    return np.asarray(blocks, np.float32).reshape(-1, 3, 3).transpose(0, 2, 1)


def _mul(a, b):
    """3x3 products with each entry summed left to right in float32."""
    out = np.zeros(np.broadcast_shapes(a.shape, b.shape), np.float32)
    for i in range(3):
        for j in range(3):
            acc = np.zeros(out.shape[:-2], np.float32)
            for k in range(3):
                acc = acc + a[..., i, k] * b[..., k, j]
            out[..., i, j] = acc
    return out


def chol_inv(a):
    """Inverse of the lower Cholesky factor of each SPD 3x3 block, with the
    diagonal fallback of a non-positive pivot (as the kernel k_chol_inv)."""
    a = a.astype(np.float32)
    l00 = np.sqrt(a[:, 0, 0])
    l10, l20 = a[:, 1, 0] / l00, a[:, 2, 0] / l00
    d1 = a[:, 1, 1] - l10 * l10
    l11 = np.sqrt(np.maximum(d1, 0))
    l21 = (a[:, 2, 1] - l20 * l10) / l11
    d2 = a[:, 2, 2] - l20 * l20 - l21 * l21
    l22 = np.sqrt(np.maximum(d2, 0))
    i00, i11, i22 = 1 / l00, 1 / l11, 1 / l22
    i10 = -l10 * i00 * i11
    i21 = -l21 * i11 * i22
    i20 = -(l20 * i00 + l21 * i10) * i22
    c = np.zeros_like(a)
    c[:, 0, 0], c[:, 1, 0], c[:, 1, 1] = i00, i10, i11
    c[:, 2, 0], c[:, 2, 1], c[:, 2, 2] = i20, i21, i22
    bad = ~((a[:, 0, 0] > 0) & (d1 > 0) & (d2 > 0) & np.isfinite(l22))
    if bad.any():
        c[bad] = 0
        for k in range(3):
            c[bad, k, k] = 1 / np.sqrt(np.maximum(np.abs(a[bad, k, k]), 1e-30))
    return c


def transpose_list(n, off, col):
    """(tr_off, tr): for each column c, the (row, slot) of every upper entry
    (row, c) with row != c, in increasing slot order."""
    off = np.asarray(off, np.int64)
    col = np.asarray(col, np.int64)
    row = np.repeat(np.arange(n), np.diff(off))
    keep = np.nonzero(row != col)[0]
    order = keep[np.argsort(col[keep], kind="stable")]
    cnt = np.bincount(col[order], minlength=n)
    tr_off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.uint32)
    tr = np.stack([row[order], order], 1).astype(np.uint32)
    return tr_off, tr


class Graph:
    """A Newton system as the network's graph.

    fixed: (off, col, val) of the fixed pattern's upper CSR (diagonal blocks
    included, 9 column-major floats per block); contact: the same for the
    contact blocks outside the pattern (no diagonal); dof_mask: nonzero for a
    Dirichlet vertex; mass per vertex. Neighbours of a vertex are visited in
    the kernels' order: fixed upper entries, fixed transposed entries, contact
    upper entries, contact transposed entries, skipping Dirichlet vertices."""

    def __init__(self, n, fixed, contact, dof_mask, mass):
        self.n = n
        self.dof = np.asarray(dof_mask, np.uint32)
        self.mass = np.asarray(mass, np.float32)
        f_off, f_col, f_val = (np.asarray(a) for a in fixed)
        c_off, c_col, c_val = (np.asarray(a) for a in contact)
        self.nnz_f = int(f_off[-1])
        self.nnz_c = int(c_off[-1])
        f_row = np.repeat(np.arange(n), np.diff(f_off.astype(np.int64)))
        c_row = np.repeat(np.arange(n), np.diff(c_off.astype(np.int64)))
        self.parts = [
            (f_off.astype(np.int64), f_col.astype(np.int64), _cols(f_val), f_row),
            (c_off.astype(np.int64), c_col[:self.nnz_c].astype(np.int64),
             _cols(c_val[:9 * self.nnz_c]), c_row),
        ]
        self.tr = [transpose_list(n, f_off, f_col), transpose_list(n, c_off, c_col[:self.nnz_c])]
        dslot = np.nonzero(f_row == f_col.astype(np.int64))[0]
        self.diag_slot = np.zeros(n, np.int64)
        self.diag_slot[f_row[dslot]] = dslot
        self.A_ii = self.parts[0][2][self.diag_slot]
        self.cinv = chol_inv(self.A_ii)
        # edges: every upper off-diagonal entry; edge index = slot (fixed) or
        # nnz_f + slot (contact)
        lo = np.concatenate([f_row, c_row])
        hi = np.concatenate([f_col, c_col[:self.nnz_c]]).astype(np.int64)
        blk = np.concatenate([self.parts[0][2], self.parts[1][2]])
        self.lo, self.hi = lo, hi
        self.part = np.concatenate([np.zeros(self.nnz_f, np.int64), np.ones(self.nnz_c, np.int64)])
        self.live = (lo != hi) & (self.dof[lo] == 0) & (self.dof[hi] == 0)
        # Â(hi, lo) = (C_hi A(hi, lo)) C_lo^T, A(hi, lo) = (upper block)^T
        ah = _mul(_mul(self.cinv[hi], blk.transpose(0, 2, 1)), self.cinv[lo].transpose(0, 2, 1))
        self.ah = np.where(self.live[:, None, None], ah, 0).astype(np.float32)
        # neighbour lists in visiting order
        nbr = [[] for _ in range(n)]
        for p in range(2):
            off, col, _, row = self.parts[p]
            base = 0 if p == 0 else self.nnz_f
            tr_off, tr = self.tr[p]
            for i in range(n):
                if self.dof[i]:
                    continue
                for k in range(off[i], off[i + 1]):
                    j = col[k]
                    if j != i and not self.dof[j]:
                        nbr[i].append((j, base + k))
                for t in range(tr_off[i], tr_off[i + 1]):
                    r, k = int(tr[t, 0]), int(tr[t, 1])
                    if not self.dof[r]:
                        nbr[i].append((r, base + k))
        self.deg = np.array([len(a) for a in nbr], np.int64)
        m = max(1, int(self.deg.max()) if n else 1)
        self.nbr = np.full((n, m), -1, np.int64)
        self.nbr_edge = np.full((n, m), -1, np.int64)
        for i, a in enumerate(nbr):
            if a:
                self.nbr[i, :len(a)] = [x[0] for x in a]
                self.nbr_edge[i, :len(a)] = [x[1] for x in a]
        self.free = self.dof == 0
        self.n_free = int(self.free.sum())

    def seq_sum(self, vals):
        """sum over each vertex's neighbours, left to right in float32:
        vals [n, ...] indexed by neighbour."""
        acc = np.zeros((self.n,) + vals.shape[1:], np.float32)
        for k in range(self.nbr.shape[1]):
            j = self.nbr[:, k]
            ok = j >= 0
            acc[ok] = acc[ok] + vals[j[ok]]
        return acc

    def node_features(self):
        """X0: the diagonal block over its mean diagonal entry (9, column-major),
        0.1 ln(mean diagonal / mass), contact neighbours / 8, sum and sum of
        squares of |Â(i, j)|_F over the neighbours, fixed-pattern neighbours /
        16, 0, and the bias column."""
        n = self.n
        X = np.zeros((n, IN0), np.float32)
        a = self.A_ii
        s = ((a[:, 0, 0] + a[:, 1, 1]) + a[:, 2, 2]) / np.float32(3)
        X[:, 0:9] = (a.transpose(0, 2, 1).reshape(n, 9) / s[:, None]).astype(np.float32)
        ratio = np.where(self.mass > 0, s / np.where(self.mass > 0, self.mass, 1), 1).astype(np.float32)
        X[:, 9] = np.float32(0.1) * np.log(ratio).astype(np.float32)
        nrm = _fro(self.ah)
        cnt_c = np.zeros(n, np.float32)
        cnt_f = np.zeros(n, np.float32)
        s1 = np.zeros(n, np.float32)
        s2 = np.zeros(n, np.float32)
        for k in range(self.nbr.shape[1]):
            e = self.nbr_edge[:, k]
            ok = e >= 0
            ee = e[ok]
            s1[ok] = s1[ok] + nrm[ee]
            s2[ok] = s2[ok] + nrm[ee] * nrm[ee]
            cnt_c[ok] += (self.part[ee] == 1)
            cnt_f[ok] += (self.part[ee] == 0)
        X[:, 10] = cnt_c / np.float32(8)
        X[:, 11] = s1
        X[:, 12] = s2
        X[:, 13] = cnt_f / np.float32(16)
        X[~self.free, :15] = 0
        X[:, 15] = 1
        return bf16(X)

    def edge_features(self):
        E = len(self.lo)
        F = np.zeros((E, INF), np.float32)
        F[:, 0:9] = self.ah.transpose(0, 2, 1).reshape(E, 9)
        F[:, 9] = _fro(self.ah)
        F[:, 10] = 1
        F[~self.live] = 0
        return bf16(F)


def _fro(m):
    m = m.reshape(len(m), 9).astype(np.float32)
    acc = np.zeros(len(m), np.float32)
    for e in range(9):
        acc = acc + m[:, e] * m[:, e]
    return np.sqrt(acc)


def _mm(a, b):
    """fp32-accumulated product of bf16-valued float32 matrices."""
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(np.float32)


# ---- network ------------------------------------------------------------------------


def forward(g: Graph, w):
    """All intermediate arrays of the network on graph g with weight blob w
    (float32 values of the bf16 weights)."""
    v = weight_views(bf16(w))
    out = {"X0": g.node_features(), "F": g.edge_features()}
    Hs = [bf16(np.maximum(_mm(out["X0"], v["W0"].T), 0))]
    Xs = []
    inv = np.where(g.deg > 0, g.deg, 1).astype(np.float32)
    for l in range(3):
        h = Hs[-1]
        mean = np.where(g.deg[:, None] > 0, g.seq_sum(h) / inv[:, None], 0).astype(np.float32)
        X = np.zeros((g.n, INL), np.float32)
        X[:, :32], X[:, 32:64], X[:, 64] = h, bf16(mean), 1
        Xs.append(X)
        Hs.append(bf16(np.maximum(_mm(X, v["W" + str(l + 1)].T), 0)))
    Xh = np.zeros((g.n, INH), np.float32)
    Xh[:, :32], Xh[:, 32] = Hs[-1], 1
    Y = _mm(Xh, v["Wh"].T)
    out.update(H=Hs, X=Xs, Xh=Xh, Y=Y)
    # edge head
    t = _mm(out["F"], v["Wf"].T)
    z = np.maximum((Y[g.hi, :32] + Y[g.lo, 32:64]) + t, 0).astype(np.float32)
    o = _mm(z, v["wo"][:32, None])[:, 0] + v["wo"][32]
    alpha = (2.0 / (1.0 + np.exp(-o.astype(np.float64)))).astype(np.float32)
    alpha[~g.live] = 0
    q = Y[:, 64]
    d = np.exp(np.clip(q, -CLAMP_Q, CLAMP_Q).astype(np.float64)).astype(np.float32)
    out.update(z=z, o=o, alpha=alpha, q=q, d=d)
    return out


def _gt_apply(g, alpha, d, w):
    """u = Ĝ^T w for probes w [W, n, 3]."""
    u = d[None, :, None] * w
    lv = np.nonzero(g.live)[0]
    contrib = -alpha[lv][None, :, None] * np.einsum("eji,wej->wei", g.ah[lv], w[:, g.hi[lv]])
    np.add.at(u, (slice(None), g.lo[lv]), contrib)
    return u


def _ahat_apply(g, u):
    """v = Â u (Dirichlet rows and columns dropped)."""
    aii = _mul(_mul(g.cinv, g.A_ii), g.cinv.transpose(0, 2, 1))
    v = np.einsum("nij,wnj->wni", aii, u) * g.free[None, :, None]
    lv = np.nonzero(g.live)[0]
    np.add.at(v, (slice(None), g.hi[lv]), np.einsum("eij,wej->wei", g.ah[lv], u[:, g.lo[lv]]))
    np.add.at(v, (slice(None), g.lo[lv]), np.einsum("eji,wej->wei", g.ah[lv], u[:, g.hi[lv]]))
    return v


def loss(g: Graph, alpha, d, probes):
    """Kaporin loss of the factor (alpha, d) with probes [W, n, 3] (Dirichlet
    vertices' entries are ignored); returns (L, T, u, v) in float64."""
    w = probes.astype(np.float64) * g.free[None, :, None]
    u = _gt_apply(g, alpha.astype(np.float64), d.astype(np.float64), w)
    v = _ahat_apply(g, u)
    W = w.shape[0]
    T = float((u * v).sum() / W)
    N = 3 * g.n_free
    L = np.log(T / N) - 2.0 / g.n_free * float(np.log(d[g.free].astype(np.float64)).sum())
    return L, T, u, v


def loss_and_grad(g: Graph, w, probes):
    """Kaporin loss and its gradient with respect to the weight blob, through
    the same bf16 rounding points as the kernels' backward pass."""
    f = forward(g, w)
    v_w = weight_views(bf16(w))
    L, T, u, v = loss(g, f["alpha"], f["d"], probes)
    W = probes.shape[0]
    c = 2.0 / (W * T)
    pw = probes.astype(np.float64) * g.free[None, :, None]
    # d L / d alpha_e = -c sum_w w_hi^T Â(hi, lo) v_lo
    galpha = -c * np.einsum("wei,eij,wej->e", pw[:, g.hi], g.ah.astype(np.float64), v[:, g.lo])
    galpha[~g.live] = 0
    al = f["alpha"].astype(np.float64)
    go = (galpha * al * (1 - al / 2)).astype(np.float32)
    go[~g.live] = 0
    # d L / d q_i = d_i c sum_w w_i . v_i - 2 / n_free  (zero where q is clamped)
    wv = np.einsum("wni,wni->n", pw, v)
    gq = f["d"].astype(np.float64) * c * wv - 2.0 / g.n_free
    gq[(np.abs(f["q"]) > CLAMP_Q) | ~g.free] = 0
    gq = gq.astype(np.float32)
    grad = np.zeros(N_WEIGHTS, np.float32)
    gv = weight_views(grad)
    # edge head
    z = f["z"]
    gz = (go[:, None] * v_w["wo"][None, :32] * (z > 0)).astype(np.float32)
    gv["wo"][:32] = _mm(go[None, :], z)[0]
    gv["wo"][32] = go.astype(np.float64).sum()
    gv["Wf"][...] = _mm(bf16(gz).T, f["F"])
    gY = np.zeros((g.n, OUTH), np.float32)
    # per vertex, summed over its neighbours in visiting order: an edge adds
    # its gz to Y[hi, 0:32] and to Y[lo, 32:64]
    for k in range(g.nbr.shape[1]):
        e = g.nbr_edge[:, k]
        ok = e >= 0
        rows = np.nonzero(ok)[0]
        ee = e[ok]
        as_hi = g.hi[ee] == rows
        gY[rows[as_hi], 0:32] = gY[rows[as_hi], 0:32] + gz[ee[as_hi]]
        gY[rows[~as_hi], 32:64] = gY[rows[~as_hi], 32:64] + gz[ee[~as_hi]]
    gY[:, 64] = gq
    gYb = bf16(gY)
    gv["Wh"][...] = _mm(gYb.T, f["Xh"])
    gXh = _mm(gYb, v_w["Wh"])
    gH = gXh[:, :32]
    inv = np.where(g.deg > 0, g.deg, 1).astype(np.float32)
    for l in (3, 2, 1):
        gZ = bf16(gH * (f["H"][l] > 0))
        X = f["X"][l - 1]
        gv["W" + str(l)][...] = _mm(gZ.T, X)
        gX = _mm(gZ, v_w["W" + str(l)])
        scaled = (gX[:, 32:64] / inv[:, None]).astype(np.float32)
        scaled[g.deg == 0] = 0
        gH = gX[:, :32] + g.seq_sum(scaled)
    gZ0 = bf16(gH * (f["H"][0] > 0))
    gv["W0"][...] = _mm(gZ0.T, f["X0"])
    return L, grad, f


def factor_dense(g: Graph, alpha, d):
    """Ĝ as a dense (3n x 3n) matrix in the normalised space (small cases)."""
    n = g.n
    G = np.zeros((3 * n, 3 * n))
    for i in range(n):
        G[3 * i:3 * i + 3, 3 * i:3 * i + 3] = (d[i] if g.free[i] else 1.0) * np.eye(3)
    for e in np.nonzero(g.live)[0]:
        hi, lo = g.hi[e], g.lo[e]
        G[3 * hi:3 * hi + 3, 3 * lo:3 * lo + 3] = -alpha[e] * g.ah[e]
    return G
