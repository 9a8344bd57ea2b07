"""The aggregate additive-Schwarz preconditioner (ParamSet::precond == 1).

CPU: the product's aggregation equals the oracle's restatement of the
reference's heavy-edge aggregation on seeded graphs, with every aggregate at
most kmax vertices and connected in the graph.

GPU: a Schwarz-preconditioned solve solves the oracle's Newton system to the
same relative residual as block-Jacobi in fewer iterations; a trajectory run
with it keeps the invariants; one step from an identical state agrees with
the oracle's block-Jacobi step within 1e-5 relative.
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
