"""The traversal autotuner (ppf_autotune, ppf_get_tuning, ppf_set_tuning).

Each traversal kernel tests the leaves of its stackless walk in warp rounds
or on the spot; the two forms must find the same pairs and the same times of
impact, so the choice is free for speed. GPU: on the two-sheet scene (every
contact kind) and the rods-and-sheet scene, the first Newton system's pair
lists are the same sets under both forms of every kernel, and the contact
line search returns the same time of impact bit for bit; the autotuner
returns a valid choice and the scene steps under it.
"""
import ctypes as C

import numpy as np
import pytest

import step_scenes
from ppf_gb300.session import Session

ALL_ROUNDS = (0, 0, 0, 0, 0, 0)
ALL_SPOT = (1, 1, 1, 1, 1, 1)


def _set(lib, modes):
    lib.ppf_set_tuning.argtypes = [C.POINTER(C.c_ubyte)]
    m = (C.c_ubyte * 6)(*modes)
    assert lib.ppf_set_tuning(m) == 0


def _pairs(lib, sc):
    from oracle.binding import product_system

    n = sc.vertex_count
    dx = np.zeros(3 * n, np.float32)
    it, rr = C.c_uint(), C.c_float()
    assert lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr)) == 0
    sysm = product_system(lib, n)
    return {k: sorted(map(tuple, sysm[k].tolist())) for k in ("pf", "pe", "pp", "ee")}


def _line_search(lib, x0, x1):
    lib.ppf_debug_contact_line_search.restype = C.c_float
    lib.ppf_debug_contact_line_search.argtypes = [C.POINTER(C.c_float)] * 2 + [
        C.POINTER(C.c_uint)]
    ov = C.c_uint()
    a = np.ascontiguousarray(x0, np.float32).reshape(-1)
    b = np.ascontiguousarray(x1, np.float32).reshape(-1)
    t = lib.ppf_debug_contact_line_search(a.ctypes.data_as(C.POINTER(C.c_float)),
                                          b.ctypes.data_as(C.POINTER(C.c_float)), C.byref(ov))
    return t, ov.value


@pytest.mark.gpu
@pytest.mark.parametrize("make", [step_scenes.two_sheets, step_scenes.rods_and_sheet])
def test_leaf_test_forms_agree(product_lib, make):
    """Pair sets equal, and the contact line search's time of impact equal
    bit for bit, under either form of every kernel: the Newton direction of
    the first system and a sweep that drives the upper object through the
    lower one."""
    lib = product_lib
    sc, _ = make()
    n = sc.vertex_count
    x0 = sc.positions()[0].copy()
    order = sc.array("vertex_order")
    s = Session(sc)
    # one Newton direction for both forms (two solves would differ by the
    # order of the assembly's atomic sums)
    _set(lib, ALL_ROUNDS)
    dx = np.zeros(3 * n, np.float32)
    it, rr = C.c_uint(), C.c_float()
    lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr))
    xd = np.empty_like(x0)
    xd[order] = x0  # the DataSet's vertex order
    down = xd.copy()
    down[:, 1] -= 4e-3 * np.linspace(0.0, 1.0, n)
    res = {}
    for modes in (ALL_ROUNDS, ALL_SPOT):
        _set(lib, modes)
        res[modes] = _pairs(lib, sc)
        res[modes, "ls"] = (_line_search(lib, xd, xd - dx.reshape(-1, 3)),
                            _line_search(lib, xd, down))
    a, b = res[ALL_ROUNDS], res[ALL_SPOT]
    assert sum(len(v) for v in a.values()) > 0
    for k in a:
        assert a[k] == b[k], k
    assert res[ALL_ROUNDS, "ls"] == res[ALL_SPOT, "ls"], (res[ALL_ROUNDS, "ls"],
                                                         res[ALL_SPOT, "ls"])
    assert res[ALL_ROUNDS, "ls"][1][0] < 1.0  # the sweep meets a contact
    _set(lib, (0, 1, 0, 0, 0, 0))
    del s


@pytest.mark.gpu
def test_autotune_choice_is_valid(product_lib):
    lib = product_lib
    sc, _ = step_scenes.two_sheets()
    s = Session(sc)
    lib.ppf_autotune.argtypes = [C.POINTER(C.c_ubyte)]
    m = (C.c_ubyte * 6)()
    assert lib.ppf_autotune(m) == 0
    modes = list(m)
    assert all(v in (0, 1) for v in modes)
    g = (C.c_ubyte * 6)()
    lib.ppf_get_tuning.argtypes = [C.POINTER(C.c_ubyte)]
    lib.ppf_get_tuning(g)
    assert list(g) == modes
    for _ in range(3):
        assert s.step().success()
    _set(lib, (0, 1, 0, 0, 0, 0))  # the defaults back for the tests after this one
