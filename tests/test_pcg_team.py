"""The PCG on one thread-block cluster against the whole grid.

Each solve is one persistent launch: over the whole grid (grid barriers
through L2) or as one cluster of up to 16 CTAs (the cluster's hardware
barrier). The recurrence is the same; only the fold of the per-block
partial sums differs (16 against 152 partials), so the two stop within a
few iterations of each other and solve the system to the same tolerance.
"""
import ctypes as C

import numpy as np
import pytest

import step_scenes
from ppf_gb300 import scenes
from ppf_gb300.session import Session

pytestmark = pytest.mark.gpu

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


def _apply(sysm, v):
    """y = A v in float64: the fixed upper pattern (per-vertex diagonal
    folded in) and the contact blocks, each with its transpose below the
    diagonal; blocks column-major."""
    v = np.asarray(v, np.float64).reshape(-1, 3)
    n = len(v)
    y = np.zeros((n, 3))
    for off, col, val in ((sysm["f_off"], sysm["f_col"], sysm["f_val"]),
                          (sysm["d_off"], sysm["d_col"], sysm["d_val"])):
        rows = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
        cols = col.astype(np.int64)
        B = val.astype(np.float64).reshape(-1, 3, 3).transpose(0, 2, 1)
        np.add.at(y, rows, np.einsum("kij,kj->ki", B, v[cols]))
        lower = rows != cols
        np.add.at(y, cols[lower], np.einsum("kji,kj->ki", B[lower], v[rows[lower]]))
    return y.reshape(-1)


@pytest.fixture
def lib(oracle_lib, product_lib):
    product_lib.ppf_set_pcg_team.argtypes = [C.c_int]
    yield product_lib
    product_lib.ppf_set_pcg_team(-1)


def test_team_sizes_and_default(lib):
    sc, _ = scenes.cloth_sphere(16)
    Session(sc)
    small = lib.ppf_pcg_team()
    assert small >= 2  # 256 vertices: one cluster
    assert lib.ppf_set_pcg_team(17) == -1
    assert lib.ppf_set_pcg_team(small + 1) == (0 if small < 16 else -1)
    assert lib.ppf_set_pcg_team(0) == 0 and lib.ppf_pcg_team() == 0
    assert lib.ppf_set_pcg_team(2) == 0 and lib.ppf_pcg_team() == 2
    assert lib.ppf_set_pcg_team(-1) == 0 and lib.ppf_pcg_team() == small
    sc, _ = scenes.cloth_sphere(130)  # 16,900 vertices: the whole grid
    Session(sc)
    assert lib.ppf_pcg_team() == 0


def test_cluster_and_grid_solve_the_same_system(lib):
    from oracle import binding

    sc, _ = step_scenes.two_sheets()
    n = sc.vertex_count
    Session(sc)
    dx = np.empty(3 * n, np.float32)
    it, rr = C.c_uint(), C.c_float()
    assert lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr)) == 0
    sysm = binding.product_system(lib, n)
    assert sysm["d_col"].size > 0
    b = sysm["force"].astype(np.float32).reshape(-1)
    lib.ppf_debug_pcg.argtypes = [f32p, f32p, C.c_uint, C.POINTER(C.c_uint),
                                  C.POINTER(C.c_float)]
    big = 16
    while lib.ppf_set_pcg_team(big) != 0:
        big //= 2
    assert big >= 2
    xs, its = [], []
    for team in (0, big, 2):
        assert lib.ppf_set_pcg_team(team) == 0
        x = np.zeros_like(b)
        st = lib.ppf_debug_pcg(b, x, 10000, C.byref(it), C.byref(rr))
        assert st == 0 and rr.value < 1e-3, (team, st, rr.value)
        r = b.astype(np.float64) - _apply(sysm, x)
        assert np.abs(r).sum() / np.abs(b).sum() < 2e-3, team
        xs.append(x.astype(np.float64))
        its.append(it.value)
    # one cluster of smaller CTAs (several solves can then share an SM)
    lib.ppf_set_pcg_cta_threads.argtypes = [C.c_uint]
    assert lib.ppf_set_pcg_cta_threads(300) == -1
    for threads in (256, 512):
        assert lib.ppf_set_pcg_cta_threads(threads) == 0
        assert lib.ppf_set_pcg_team(big) == 0
        x = np.zeros_like(b)
        st = lib.ppf_debug_pcg(b, x, 10000, C.byref(it), C.byref(rr))
        assert st == 0 and rr.value < 1e-3, (threads, st, rr.value)
        r = b.astype(np.float64) - _apply(sysm, x)
        assert np.abs(r).sum() / np.abs(b).sum() < 2e-3, threads
        xs.append(x.astype(np.float64))
        its.append(it.value)
    assert lib.ppf_set_pcg_cta_threads(0) == 0
    for x in xs[1:]:
        assert np.linalg.norm(x - xs[0]) / np.linalg.norm(xs[0]) < 2e-2, its
    assert max(its) <= 1.2 * min(its) + 4, its


def test_cluster_and_grid_steps_agree(lib):
    runs = []
    for team in (0, -1):
        assert lib.ppf_set_pcg_team(team) == 0
        sc, _ = scenes.cloth_sphere(24)
        s = Session(sc)
        assert lib.ppf_pcg_team() == (0 if team == 0 else lib.ppf_pcg_team())
        for _ in range(10):
            assert s.step().success()
        runs.append(s.positions())
    assert np.abs(runs[0] - runs[1]).max() <= 1e-5 * np.abs(runs[1]).max()
