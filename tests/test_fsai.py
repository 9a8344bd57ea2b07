"""The FSAI factor of the factored preconditioner (csrc/gpu/fsai.cu).

CPU: the oracle's factor has the FSAI properties ((Ĝ Â Ĝ^T)(i, i) = I and
(Ĝ Â)(i, j) = 0 on each row's pattern), keeps the strongest couplings of a
row with too many, and preconditions CG better than block-Jacobi.
GPU: the solver's factor against the oracle's on the same Newton system, the
factored solve against the system, and trajectory invariants.
"""
import ctypes as C

import numpy as np
import pytest

import learned_cases
from oracle import fsai as OF
from oracle import learned as OL


def _pcg_iters(A, b, apply_p, tol=1e-3, maxit=5000):
    x = np.zeros_like(b)
    r = b.copy()
    err0 = np.abs(r).sum()
    z = apply_p(r)
    p = z.copy()
    rz = r @ z
    for it in range(1, maxit + 1):
        Ap = A @ p
        a = rz / (p @ Ap)
        x += a * p
        r -= a * Ap
        if np.abs(r).sum() / err0 < tol:
            return it
        z = apply_p(r)
        rz1 = r @ z
        p = z + rz1 / rz * p
        rz = rz1
    return maxit


def test_oracle_fsai_properties():
    s = learned_cases.synthetic(n=80, seed=3, hub=30)
    g = learned_cases.graph(s)
    gdiag, gedge, kept = OF.factor(g)
    G = OF.dense_factor(g, gdiag, gedge)
    A = OF.dense_operator(g)
    # the factor is built from the float32 normalised blocks: its properties
    # hold to float32 rounding of those blocks
    M = G @ A @ G.T
    GA = G @ A
    for i in range(g.n):
        if not g.free[i]:
            continue
        np.testing.assert_allclose(M[3 * i:3 * i + 3, 3 * i:3 * i + 3], np.eye(3), atol=1e-6)
        for v, _ in kept[i]:
            assert np.abs(GA[3 * i:3 * i + 3, 3 * v:3 * v + 3]).max() < 1e-6
    # the hub row keeps its 15 strongest lower couplings
    hub = g.n - 1
    assert len(kept[hub]) == OF.MAX_LOWER
    lower = [(int(g.lo[e]), e) for e in range(len(g.lo)) if g.hi[e] == hub and g.live[e]]
    norms = sorted((float(OL._fro(g.ah[e:e + 1])[0]) for _, e in lower), reverse=True)
    got = sorted((float(OL._fro(g.ah[e:e + 1])[0]) for _, e in kept[hub]), reverse=True)
    assert got == norms[:OF.MAX_LOWER]


def test_oracle_fsai_preconditions_better_than_block_jacobi():
    s = learned_cases.synthetic(n=300, seed=5)
    g = learned_cases.graph(s)
    gdiag, gedge, _ = OF.factor(g)
    G = OF.dense_factor(g, gdiag, gedge)
    A = OF.dense_operator(g)
    free = np.repeat(g.free, 3)
    b = np.random.default_rng(1).normal(size=3 * g.n) * free
    D = np.zeros_like(A)
    for i in range(g.n):
        D[3 * i:3 * i + 3, 3 * i:3 * i + 3] = np.linalg.inv(A[3 * i:3 * i + 3, 3 * i:3 * i + 3])
    it_bj = _pcg_iters(A, b, lambda r: D @ r)
    it_f = _pcg_iters(A, b, lambda r: G.T @ (G @ r) + 1e-3 * (D @ r))
    assert it_f < it_bj, (it_f, it_bj)


# ---- GPU ----------------------------------------------------------------------------------------


def _debug_solve(lib, n):
    dx = np.empty(3 * n, np.float32)
    it, rr = C.c_uint(), C.c_float()
    st = lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr))
    return st, dx.reshape(-1, 3), it.value, rr.value


@pytest.mark.gpu
def test_gpu_fsai_factor_matches_oracle(product_lib):
    """Two sheets in contact, pinned corners: G(i, i) of the solver's FSAI
    factor against the oracle's on the same Newton system, and the factored
    solve against that system."""
    import step_scenes
    from ppf_gb300 import abi
    from ppf_gb300 import learned as PL
    from ppf_gb300.session import Session
    from test_step_parity import _apply

    sc, _ = step_scenes.two_sheets()
    n = sc.vertex_count
    s = Session(sc)
    s.set_preconditioner(abi.PRECOND_FIRST_ORDER, 0.5)
    _, _, it_fo, _ = _debug_solve(product_lib, n)
    s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
    _, _, it_bj, _ = _debug_solve(product_lib, n)
    s.set_preconditioner(abi.PRECOND_FSAI)
    st, dx, it_f, rr = _debug_solve(product_lib, n)
    sysd = PL.capture_system(n)  # the same state: the same system, solved again
    diag = np.zeros(9 * n, np.float32)
    PL.lib().ppf_debug_factor_diag(diag)
    s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
    g = learned_cases.graph(sysd)
    gdiag, gedge, kept = OF.factor(g)
    assert sum(len(v) for v in kept.values()) > n  # contact and fixed couplings kept
    Gd = diag.reshape(n, 3, 3).transpose(0, 2, 1)
    err = np.abs(Gd - gdiag).max() / np.abs(gdiag).max()
    assert err < 1e-3, err
    assert st == 0 and rr < 1e-3
    so = {"f_off": sysd["f_off"], "f_col": sysd["f_col"], "f_val": sysd["f_val"].reshape(-1, 9),
          "d_off": sysd["d_off"], "d_col": sysd["d_col"], "d_val": sysd["d_val"].reshape(-1, 9)}
    bvec = sysd["force"].astype(np.float64).reshape(-1)
    res = np.abs(bvec - _apply(so, dx)).sum() / np.abs(bvec).sum()
    assert res < 2e-3, res
    assert it_f < it_fo < it_bj, (it_f, it_fo, it_bj)


@pytest.mark.gpu
def test_fsai_on_a_held_out_scene(product_lib):
    """Stacked sheets of 8 x 64^2: PCG iterations and time of the same steps
    with block-Jacobi and with the FSAI factor."""
    from ppf_gb300 import abi, scenes
    from ppf_gb300.session import Session

    out = {}
    for name, kind in (("block_jacobi", abi.PRECOND_BLOCK_JACOBI), ("fsai", abi.PRECOND_FSAI)):
        sc, _ = scenes.stacked_sheets(side=64, sheets=8, seed=11)
        s = Session(sc)
        s.set_preconditioner(kind)
        it = fb = 0
        ms = 0.0
        for _ in range(30):
            assert s.step(fetch=False).success()
            st = s.stats()
            it += st.pcg_iters_total
            fb += st.fallbacks
            ms += st.pcg_ms_total
        s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
        out[name] = (it, fb, round(ms, 1))
    print(f"\nheld-out stacked sheets 64x8, 30 steps (PCG iterations, fallbacks, ms): {out}")
    assert out["fsai"][0] < 0.6 * out["block_jacobi"][0], out


@pytest.mark.gpu
def test_fsai_trajectory_invariants(product_lib, oracle_lib):
    from oracle.binding import OracleSession
    from ppf_gb300 import abi, scenes
    from ppf_gb300.session import Session

    sc, _ = scenes.cloth_sphere(24)
    s = Session(sc)
    s.set_preconditioner(abi.PRECOND_FSAI)
    orc = OracleSession(sc)
    for step in range(40):
        assert s.step().success()
        if step % 8 == 7:
            assert orc.intersection_free(s.positions())
    assert s.stats().precond_kind == abi.PRECOND_FSAI
    s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
