"""The factored preconditioner P = G^T G + eps D^{-1} of the PCG (GPU).

The factored solve must solve the same Newton system as block-Jacobi does,
to the same relative residual (checked against the oracle's system in
float64), in fewer iterations on contact-coupled systems; and a trajectory
run with it keeps the same invariants as the block-Jacobi one.
"""
import ctypes as C

import numpy as np
import pytest

import step_scenes
from ppf_gb300 import abi, scenes
from ppf_gb300.session import Session

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def binding(oracle_lib, product_lib):
    from oracle import binding

    return binding


def _debug_solve(lib, n):
    dx = np.empty(3 * n, np.float32)
    it, rr = C.c_uint(), C.c_float()
    st = lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr))
    return st, dx.reshape(-1, 3), it.value, rr.value


def test_first_order_factor_solves_the_system_in_fewer_iterations(binding, product_lib):
    from test_step_parity import _apply

    sc, _ = step_scenes.two_sheets()
    n = sc.vertex_count
    orc = binding.OracleSession(sc)
    orc.newton_system()
    so = orc.system()
    s = Session(sc)
    s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
    st_j, dx_j, it_j, _ = _debug_solve(product_lib, n)
    s = Session(sc)
    s.set_preconditioner(abi.PRECOND_FIRST_ORDER, 0.5)
    st_f, dx_f, it_f, rr_f = _debug_solve(product_lib, n)
    s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
    assert st_j == 0 and st_f == 0 and rr_f < 1e-3
    b = so["force"].astype(np.float64).reshape(-1)
    res = np.abs(b - _apply(so, dx_f)).sum() / np.abs(b).sum()
    assert res < 2e-3, res
    assert it_f < it_j, (it_f, it_j)


def test_first_order_factor_trajectory_invariants(binding):
    sc, _ = scenes.cloth_sphere(24)
    rest = sc.positions()[0].copy()
    from ppf_gb300 import meshes

    _, faces = meshes.grid(24, 24)
    s = Session(sc)
    s.set_preconditioner(abi.PRECOND_FIRST_ORDER, 0.5)
    checker = binding.OracleSession(sc)
    factor_iters = 0
    try:
        for k in range(60):
            r = s.step()
            assert r.success(), (k, r.as_dict())
            st = s.stats()
            assert st.precond_kind == abi.PRECOND_FIRST_ORDER
            factor_iters += st.factor_iters_total
            x = s.positions()
            if k % 5 == 4:
                assert checker.intersection_free(x), k
                sig = step_scenes.strain_of(x, rest, faces)
                assert sig.max() <= 1.01 + 1e-3, (k, sig.max())
    finally:
        s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
    assert factor_iters > 0
    assert np.linalg.norm(x, axis=1).min() >= 0.3 - 1e-6


def test_first_order_factor_step_matches_oracle(binding):
    """One step from an identical state with every contact kind active; the
    oracle solves with block-Jacobi, the product with the factor: both stop
    at the 1e-3 relative residual, so they agree as the block-Jacobi step
    does."""
    sc, _ = step_scenes.two_sheets()
    orc = binding.OracleSession(sc)
    for _ in range(2):
        assert orc.step().success()
    curr, prev = orc.positions()
    x0 = curr.copy()
    sc.set_positions(curr, prev)
    sc.param.contents.time = orc.time
    s = Session(sc)
    s.set_preconditioner(abi.PRECOND_FIRST_ORDER, 0.5)
    o = binding.OracleSession(sc)
    try:
        rg, ro = s.step(), o.step()
    finally:
        s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
    assert rg.success() and ro.success()
    xg, xo = s.positions(), o.positions()[0]
    err = np.abs(xg - xo).max()
    assert err <= 1e-5 * np.abs(xo).max(), (err, np.abs(xo - x0).max())
