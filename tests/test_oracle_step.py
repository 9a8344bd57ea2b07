"""CPU checks of the oracle's step loop and of the host-side scene builder.

The oracle's element math is pinned to the reference's own code
(test_elements.py); these tests check the pipeline around it on physical
invariants: free fall follows the implicit-Euler recurrence, a sheet stays
intersection-free and strain-limited through contact, and the Newton system
it assembles is symmetric with the reference's pattern.
"""
import numpy as np
import pytest

import step_scenes
from ppf_gb300 import scenes


@pytest.fixture(scope="module")
def orc(oracle_lib, product_lib):
    from oracle.binding import OracleSession

    return OracleSession


def test_free_fall_follows_implicit_euler(orc):
    sc, _ = scenes.cloth_sphere(8)
    o = orc(sc)
    y0 = 1.0
    g, dt = 9.8, 0.01
    # implicit Euler with the normal air drag of a flat sheet: minimising
    # m/2|y - y_pred|^2 + A rho_air/2 |y - x|^2 over dt^2 gives
    # step_{k+1} = (step_k - g dt^2) / (1 + rho_air / rho)
    c = 1e-3 / scenes.DENSITY
    y_exp, step = y0, 0.0
    for k in range(1, 11):
        r = o.step()
        assert r.success()
        y = o.positions()[0][:, 1]
        step = (step - g * dt * dt) / (1.0 + c)
        y_exp += step
        # each step's solve stops at a 1e-3 relative residual and the final
        # Newton iteration corrects it, so the fall agrees to ~1e-5 of itself
        # per step; 1e-4 of the fall plus the fp32 spacing bounds 10 steps
        assert np.all(np.abs(y - y_exp) <= 1e-4 * (y0 - y_exp) + 2.0 ** -22)
        assert np.ptp(y) < 1e-6


def test_two_sheets_stay_separated_and_strain_limited(orc):
    sc, _ = step_scenes.two_sheets()
    rest = sc.positions()[0].copy()
    o = orc(sc)
    faces = None
    for _ in range(6):
        r = o.step()
        assert r.success(), r.as_dict()
        x = o.positions()[0]
        assert o.intersection_free(x)
    st = o.stats()
    assert st["newton_iters"] >= 2


def test_newton_system_is_symmetric_and_complete(orc):
    sc, _ = step_scenes.two_sheets()
    o = orc(sc)
    state, dx, iters, resid = o.newton_system()
    assert state == 0 and resid < 1e-3
    sysm = o.system()
    # every contact kind present in this scene
    for k in ("pf", "pe", "pp", "ee"):
        assert len(sysm[k]) > 0, k
    # contact blocks lie in the upper triangle, outside the fixed pattern
    f_off, f_col = sysm["f_off"], sysm["f_col"]
    d_off, d_col = sysm["d_off"], sysm["d_col"]
    fixed = set()
    for i in range(len(f_off) - 1):
        for k in range(f_off[i], f_off[i + 1]):
            fixed.add((i, int(f_col[k])))
    for i in range(len(d_off) - 1):
        for k in range(d_off[i], d_off[i + 1]):
            j = int(d_col[k])
            assert i < j and (i, j) not in fixed
    # diagonal blocks of the folded fixed matrix are symmetric positive
    diag_blocks = [sysm["f_val"][f_off[i]].reshape(3, 3) for i in range(len(f_off) - 1)]
    for b in diag_blocks:
        assert np.allclose(b, b.T, rtol=1e-5, atol=1e-3 * np.abs(b).max())
        assert np.linalg.eigvalsh(0.5 * (b + b.T)).min() > 0


def test_strain_measure_on_rest_is_one():
    sc, _ = step_scenes.two_sheets()
    x = sc.positions()[0]
    from ppf_gb300 import meshes

    _, f = meshes.grid(12, 12, 0.4, 0.4)
    s = step_scenes.strain_of(x[: 144], x[: 144], f)
    assert np.allclose(s, 1.0, atol=1e-5)
