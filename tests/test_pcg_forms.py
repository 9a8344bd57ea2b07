"""The block-Jacobi PCG in its two forms on the same Newton systems, through
the C ABI: the reference's two-reduction recurrence (form 0) and the
single-reduction Chronopoulos-Gear recurrence (form 1, the default).

The forms are equal in exact arithmetic and differ by rounding, so the bar
is the one the solver itself sets: each solution's true L1 residual,
recomputed in float64 on the oracle's copy of the system, is within the
1e-3 relative tolerance (2e-3 with fp32 slack), and the iteration counts,
taken at the same check cadence, agree within a few percent.
"""
import ctypes as C

import numpy as np
import pytest

import step_scenes
from oracle import parity
from ppf_gb300 import scenes
from ppf_gb300.session import Session

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def binding(oracle_lib, product_lib):
    from oracle import binding

    product_lib.ppf_set_pcg_form.restype = C.c_int
    product_lib.ppf_set_pcg_form.argtypes = [C.c_int]
    product_lib.ppf_pcg_form.restype = C.c_int
    return binding


def _solve_both(lib, binding, sc):
    n = sc.vertex_count
    o = binding.OracleSession(sc)
    o.newton_system()
    so = o.system()
    b = so["force"].astype(np.float64).reshape(-1)
    out = {}
    for form in (0, 1):
        assert lib.ppf_set_pcg_form(form) == 0
        assert lib.ppf_pcg_form() == form
        Session(sc)
        dx = np.empty(3 * n, np.float32)
        it, rr = C.c_uint(), C.c_float()
        st = lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr))
        true = float(np.abs(b - parity.apply_system(so, dx)).sum() / np.abs(b).sum())
        out[form] = (st, it.value, rr.value, true, dx)
    lib.ppf_set_pcg_form(1)
    return out


def _check(out):
    for form, (st, it, rr, true, _) in out.items():
        assert st == 0, (form, st)
        assert rr < 1e-3, (form, rr)
        assert true < 2e-3, (form, true)
    i0, i1 = out[0][1], out[1][1]
    assert abs(i0 - i1) <= 0.05 * i0 + 4, (i0, i1)


def test_forms_agree_on_the_two_sheet_system(product_lib, binding):
    sc, _ = step_scenes.two_sheets()
    out = _solve_both(product_lib, binding, sc)
    _check(out)
    d0, d1 = out[0][4], out[1][4]
    assert np.linalg.norm(d1 - d0) <= 2e-2 * np.linalg.norm(d0)


def test_forms_agree_on_the_stacked_sheets_contact_system(product_lib, binding):
    sc, _ = scenes.stacked_sheets(128, 8, seed=0, dt=0.01)
    s = Session(sc)
    for k in range(40):
        assert s.step().success()
        if s.stats().max_dyn_blocks > 0:
            break
    out = _solve_both(product_lib, binding, sc)
    print("stacked sheets contact system: iterations", {f: v[1] for f, v in out.items()},
          "true residual", {f: v[3] for f, v in out.items()})
    _check(out)


def test_single_reduction_trajectory_invariants(product_lib, binding):
    """60 steps of a 32x32 cloth onto the sphere with the single-reduction
    form: intersection-free (the oracle's own check) and strain-limited on
    every checked frame."""
    assert product_lib.ppf_set_pcg_form(1) == 0
    sc, _ = scenes.cloth_sphere(32)
    rest = sc.positions()[0].copy()
    faces = sc.array("face").reshape(-1, 3)
    s = Session(sc)
    checker = binding.OracleSession(sc)
    for k in range(60):
        r = s.step()
        assert r.success(), (k, r.as_dict())
        if k % 4 == 3:
            x = s.positions()
            assert checker.intersection_free(x), k
            assert step_scenes.strain_of(x, rest, faces).max() <= 1.01 + 1e-3
    assert np.linalg.norm(s.positions(), axis=1).min() >= 0.3 - 1e-6
