"""The aggregate additive-Schwarz preconditioner (ParamSet::precond == 1).

CPU: the product's aggregation equals the oracle's restatement of the
reference's heavy-edge aggregation on seeded graphs, with every aggregate at
most kmax vertices and connected in the graph.

CPU: the coarse level's domains (Galerkin blocks of the aggregates grouped
by the same growth on their norms) equal the restatement's.

GPU: a Schwarz-preconditioned solve solves the oracle's Newton system to the
same relative residual as block-Jacobi in fewer iterations; a trajectory run
with it keeps the invariants; one step from an identical state agrees with
the oracle's block-Jacobi step within 1e-5 relative. On a contact system the
PCG's aggregation and coarse domains equal the restatement's bit for bit,
its first iteration is alpha P b for the restated one- and two-level
operators, and both forms solve the system to the tolerance.
"""
import ctypes as C

import numpy as np
import pytest

import step_scenes
from ppf_gb300 import abi, scenes
from ppf_gb300._lib import f32p, u32p
from ppf_gb300.session import Session


def _graph(rng, side, extra):
    """Both-triangle CSR of a grid (4-neighbour) plus random extra edges,
    with seeded positive weights (symmetric)."""
    n = side * side
    edges = set()
    for y in range(side):
        for x in range(side):
            i = y * side + x
            if x + 1 < side:
                edges.add((i, i + 1))
            if y + 1 < side:
                edges.add((i, i + side))
    for _ in range(extra):
        a, b = rng.integers(0, n, 2)
        if a != b:
            edges.add((min(a, b), max(a, b)))
    w = {e: np.float32(rng.uniform(0.1, 10.0)) for e in sorted(edges)}
    rows = [[] for _ in range(n)]
    for (a, b), v in w.items():
        rows[a].append((b, v))
        rows[b].append((a, v))
    off, col, wgt = [0], [], []
    for i in range(n):
        rows[i].append((i, np.float32(100.0)))  # the diagonal block
        for j, v in sorted(rows[i]):
            col.append(j)
            wgt.append(v)
        off.append(len(col))
    return (np.array(off, np.uint32), np.array(col, np.uint32),
            np.array(wgt, np.float32))


@pytest.mark.parametrize("seed,side,extra,kmax", [(0, 12, 0, 16), (1, 17, 40, 16),
                                                  (2, 9, 200, 5), (3, 20, 10, 1)])
def test_aggregation_matches_restatement(product_lib, seed, side, extra, kmax):
    from oracle.schwarz import hem_aggregate

    off, col, wgt = _graph(np.random.default_rng(seed), side, extra)
    n = len(off) - 1
    lib = product_lib
    lib.ppf_schwarz_aggregate.restype = C.c_uint
    lib.ppf_schwarz_aggregate.argtypes = [C.c_uint, u32p, u32p, f32p, C.c_uint, u32p]
    agg = np.zeros(n, np.uint32)
    n_agg = lib.ppf_schwarz_aggregate(n, off, col, wgt, kmax, agg)
    ref, n_ref = hem_aggregate(off, col, wgt, kmax)
    assert n_agg == n_ref
    assert np.array_equal(agg, ref)
    sizes = np.bincount(agg, minlength=n_agg)
    assert sizes.min() >= 1 and sizes.max() <= kmax
    # each aggregate is connected in the graph
    for g in range(n_agg):
        mem = set(np.nonzero(agg == g)[0].tolist())
        start = next(iter(mem))
        seen, stack = {start}, [start]
        while stack:
            v = stack.pop()
            for k in range(off[v], off[v + 1]):
                u = int(col[k])
                if u in mem and u not in seen:
                    seen.add(u)
                    stack.append(u)
        assert seen == mem, g


@pytest.fixture(scope="module")
def binding(oracle_lib, product_lib):
    from oracle import binding

    return binding


def _debug_solve(lib, n):
    dx = np.empty(3 * n, np.float32)
    it, rr = C.c_uint(), C.c_float()
    st = lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr))
    return st, dx.reshape(-1, 3), it.value, rr.value


@pytest.mark.gpu
def test_schwarz_solves_the_system_in_fewer_iterations(binding, product_lib):
    from test_step_parity import _apply

    sc, _ = step_scenes.two_sheets()
    n = sc.vertex_count
    orc = binding.OracleSession(sc)
    orc.newton_system()
    so = orc.system()
    Session(sc)
    st_j, _, it_j, _ = _debug_solve(product_lib, n)
    sc.param.contents.precond = 1
    try:
        Session(sc)
        st_s, dx_s, it_s, rr_s = _debug_solve(product_lib, n)
    finally:
        sc.param.contents.precond = 0
    assert st_j == 0 and st_s == 0 and rr_s < 1e-3
    b = so["force"].astype(np.float64).reshape(-1)
    res = np.abs(b - _apply(so, dx_s)).sum() / np.abs(b).sum()
    assert res < 2e-3, res
    assert it_s < it_j, (it_s, it_j)


@pytest.mark.gpu
def test_schwarz_trajectory_invariants(binding):
    sc, _ = scenes.cloth_sphere(24)
    sc.param.contents.precond = 1
    rest = sc.positions()[0].copy()
    from ppf_gb300 import meshes

    _, faces = meshes.grid(24, 24)
    s = Session(sc)
    checker = binding.OracleSession(sc)
    for k in range(60):
        r = s.step()
        assert r.success(), (k, r.as_dict())
        assert s.stats().precond_kind == 3
        x = s.positions()
        if k % 5 == 4:
            assert checker.intersection_free(x), k
            sig = step_scenes.strain_of(x, rest, faces)
            assert sig.max() <= 1.01 + 1e-3, (k, sig.max())
    assert np.linalg.norm(x, axis=1).min() >= 0.3 - 1e-6


@pytest.mark.gpu
def test_schwarz_step_matches_oracle(binding):
    sc, _ = step_scenes.two_sheets()
    orc = binding.OracleSession(sc)
    for _ in range(2):
        assert orc.step().success()
    curr, prev = orc.positions()
    sc.set_positions(curr, prev)
    sc.param.contents.time = orc.time
    o = binding.OracleSession(sc)
    sc.param.contents.precond = 1
    s = Session(sc)
    rg, ro = s.step(), o.step()
    assert rg.success() and ro.success()
    xg, xo = s.positions(), o.positions()[0]
    err = np.abs(xg - xo).max()
    assert err <= 1e-5 * np.abs(xo).max(), err


def _block_graph(rng, side, extra):
    """The grid graph of _graph with a seeded 3 x 3 block per entry,
    block(j, i) = block(i, j)^T (column-major, 9 floats per entry)."""
    off, col, _ = _graph(rng, side, extra)
    n = len(off) - 1
    upper = {}
    blocks = np.zeros((len(col), 9), np.float32)
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            j = int(col[k])
            key = (min(i, j), max(i, j))
            if key not in upper:
                upper[key] = rng.uniform(-1.0, 1.0, (3, 3)).astype(np.float32)
            B = upper[key] if i <= j else upper[key].T
            blocks[k] = B.T.reshape(9)  # column-major
    wgt = np.array([np.float32(np.sqrt(np.float32(np.sum(b * b)))) for b in blocks], np.float32)
    return off, col, blocks, wgt


@pytest.mark.parametrize("seed,side,extra,kmax", [(0, 16, 0, 4), (1, 21, 60, 6), (2, 12, 150, 3)])
def test_coarse_domains_match_restatement(product_lib, seed, side, extra, kmax):
    """The coarse level (Galerkin blocks of the aggregates, grouped by the
    same heavy-edge growth on their norms) equals the restatement."""
    from oracle.schwarz import galerkin_domains, hem_aggregate

    off, col, blocks, wgt = _block_graph(np.random.default_rng(seed), side, extra)
    n = len(off) - 1
    agg, n_agg = hem_aggregate(off, col, wgt, kmax)
    lib = product_lib
    lib.ppf_schwarz_coarsen.restype = C.c_uint
    lib.ppf_schwarz_coarsen.argtypes = [C.c_uint, u32p, u32p, f32p, u32p, C.c_uint, C.c_uint,
                                        u32p]
    dom = np.zeros(n_agg, np.uint32)
    n_dom = lib.ppf_schwarz_coarsen(n, off, col, blocks.reshape(-1), agg, n_agg, kmax, dom)
    ref, n_ref = galerkin_domains(off, col, blocks, agg, n_agg, kmax)
    assert n_dom == n_ref and 1 <= n_dom < n_agg
    assert np.array_equal(dom, ref)
    assert np.bincount(dom, minlength=n_dom).max() <= kmax


def _operator_rows(sysm):
    """Every off-diagonal block of each row of the product's kept system, as
    the PCG's slice layout holds it (the upper blocks and, below the
    diagonal, their transposes), sorted by column: CSR offsets, columns,
    column-major blocks and Frobenius norms in float32."""
    n = len(sysm["f_off"]) - 1
    rows = [[] for _ in range(n)]
    for off, col, val in ((sysm["f_off"], sysm["f_col"], sysm["f_val"]),
                          (sysm["d_off"], sysm["d_col"], sysm["d_val"])):
        for i in range(n):
            for k in range(off[i], off[i + 1]):
                j = int(col[k])
                if j == i:
                    continue
                v = np.asarray(val[k], np.float32)
                rows[i].append((j, v))
                rows[j].append((i, v.reshape(3, 3).T.reshape(9)))
    r_off, r_col, r_blk = [0], [], []
    for i in range(n):
        cols = [j for j, _ in rows[i]]
        assert len(cols) == len(set(cols)), i  # fixed and contact patterns are disjoint
        for j, v in sorted(rows[i], key=lambda e: e[0]):
            r_col.append(j)
            r_blk.append(v)
        r_off.append(len(r_col))
    blk = np.array(r_blk, np.float32).reshape(-1, 9)
    wgt = np.zeros(len(blk), np.float32)
    for k, b in enumerate(blk):
        w = np.float32(0.0)
        for q in range(9):
            w = np.float32(w + np.float32(b[q] * b[q]))
        wgt[k] = np.sqrt(w)
    return np.array(r_off, np.uint32), np.array(r_col, np.uint32), blk, wgt


def _full_operator(sysm):
    """The kept system as a both-triangle float64 scipy matrix (3n x 3n)."""
    import scipy.sparse as sp

    n = len(sysm["f_off"]) - 1
    R, Cc, V = [], [], []
    for off, col, val in ((sysm["f_off"], sysm["f_col"], sysm["f_val"]),
                          (sysm["d_off"], sysm["d_col"], sysm["d_val"])):
        rows = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
        cols = col.astype(np.int64)
        B = val.astype(np.float64).reshape(-1, 3, 3).transpose(0, 2, 1)  # row-major
        for a in range(3):
            for b in range(3):
                R.append(3 * rows + a)
                Cc.append(3 * cols + b)
                V.append(B[:, a, b])
                low = rows != cols
                R.append(3 * cols[low] + b)
                Cc.append(3 * rows[low] + a)
                V.append(B[low, a, b])
    return sp.csr_matrix((np.concatenate(V), (np.concatenate(R), np.concatenate(Cc))),
                         shape=(3 * n, 3 * n))


def _schwarz_system(lib, levels, side=16):
    """The first Newton system of the unpinned two-sheet scene, solved with
    the Schwarz preconditioner at `levels`; returns (scene, kept system,
    layout sizes, aggregate per vertex, domain per aggregate). The scene must
    outlive the solves that follow: the library keeps its ParamSet by
    pointer, as the reference does."""
    from oracle.binding import product_system

    sc, _ = step_scenes.two_sheets(side=side, pinned=False)
    n = sc.vertex_count
    sc.param.contents.precond = 1
    sc.param.contents.schwarz_levels = levels
    try:
        Session(sc)
        st, _, _, _ = _debug_solve(lib, n)
    finally:
        sc.param.contents.precond = 0
        sc.param.contents.schwarz_levels = 2
    assert st == 0
    sysm = product_system(lib, n)
    lib.ppf_debug_schwarz_layout.argtypes = [u32p, u32p, u32p]
    sizes = np.zeros(3, np.uint32)
    agg = np.zeros(n, np.uint32)
    dom = np.zeros(n, np.uint32)  # n_agg <= n
    lib.ppf_debug_schwarz_layout(sizes, agg, dom)
    return sc, sysm, sizes, agg, dom[:sizes[0]]


def _debug_pcg(lib, b, max_iter):
    lib.ppf_debug_pcg.argtypes = [f32p, f32p, C.c_uint, C.POINTER(C.c_uint),
                                  C.POINTER(C.c_float)]
    x = np.zeros_like(b)
    it, rr = C.c_uint(), C.c_float()
    st = lib.ppf_debug_pcg(b, x, max_iter, C.byref(it), C.byref(rr))
    return st, x, it.value, rr.value


@pytest.mark.gpu
@pytest.mark.parametrize("levels", [1, 2])
def test_schwarz_layout_and_first_direction_match_restatement(product_lib, levels):
    """On a contact system: the aggregation and (two levels) the coarse
    domains equal the restatement's on the operator the PCG holds, bit for
    bit; one PCG iteration from x = 0 gives x = alpha P b with P the
    restated one- or two-level Schwarz operator applied in float64."""
    from oracle.schwarz import galerkin_domains, hem_aggregate, schwarz_apply

    lib = product_lib
    sc, sysm, sizes, agg, dom = _schwarz_system(lib, levels)
    n = sc.vertex_count
    assert sysm["d_col"].size > 0  # contact blocks in the system
    off, col, blk, wgt = _operator_rows(sysm)
    ref_agg, n_agg = hem_aggregate(off, col, wgt, 16)
    assert sizes[0] == n_agg and np.array_equal(agg, ref_agg)
    assert sizes[2] == levels
    if levels == 2:
        ref_dom, n_dom = galerkin_domains(off, col, blk, agg, n_agg, 16)
        assert sizes[1] == n_dom and n_dom > 1
        assert np.array_equal(dom, ref_dom)
    else:
        assert sizes[1] == 0
    A = _full_operator(sysm)
    rng = np.random.default_rng(11)
    b = rng.standard_normal(3 * n).astype(np.float32)
    st, x, it, _ = _debug_pcg(lib, b, 1)
    assert it == 1
    z = schwarz_apply(A, agg, b, dom if levels == 2 else None)
    alpha = float(b.astype(np.float64) @ z) / float(z @ (A @ z))
    want = alpha * z
    err = np.abs(x - want).max() / np.abs(want).max()
    print(f"levels {levels}: first direction error {err:.2e}")
    assert err < 1e-3, err


@pytest.mark.gpu
def test_two_level_solve_reaches_tolerance(product_lib):
    """Solved to the 1e-3 relative L1 residual with one and with two levels
    on the same contact system: both solutions solve the system in float64
    to that tolerance (with float32 slack)."""
    lib = product_lib
    iters = {}
    for levels in (1, 2):
        sc, sysm, _, _, _ = _schwarz_system(lib, levels)
        A = _full_operator(sysm)
        b = sysm["force"].reshape(-1).astype(np.float32)
        st, x, it, rr = _debug_pcg(lib, b, 10000)
        assert st == 0, (levels, st, rr)
        res = np.abs(b - A @ x.astype(np.float64)).sum() / np.abs(b).sum()
        assert res < 2e-3, (levels, res)
        iters[levels] = it
    print("PCG iterations by Schwarz levels:", iters)
