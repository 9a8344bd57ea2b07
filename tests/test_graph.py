"""CUDA graphs on the Newton iteration.

* The whole iteration (assembly sized by capacities, the PCG solve, the line
  search, the status copy) runs as one replayed graph: every iteration goes
  through that path, a scene captures it once and replays it afterwards, and
  one step from an identical state matches the oracle within 1e-5 relative.
* An iteration whose pair lists or contact-block capacity were too small
  changes nothing and is repeated with grown capacities; the step it belongs
  to still matches the oracle.
* With the iteration graph off, the line-search stage alone replays as a
  graph, once per Newton iteration.
"""
import ctypes as C

import numpy as np
import pytest

import step_scenes
from ppf_gb300 import scenes
from ppf_gb300.session import Session

pytestmark = pytest.mark.gpu


def _graph_stats(lib):
    out = (C.c_ulonglong * 4)()
    lib.ppf_iteration_graph_stats(out)
    return np.array(list(out), np.int64)  # direct, captures, replays, repeats


@pytest.fixture
def lib(oracle_lib, product_lib):
    product_lib.ppf_graph_launches.restype = C.c_ulonglong
    product_lib.ppf_set_iteration_graph(1)
    yield product_lib
    product_lib.ppf_set_iteration_graph(1)


def test_line_search_stage_replays_as_a_graph(lib):
    from oracle.binding import OracleSession

    lib.ppf_set_iteration_graph(0)
    sc, _ = scenes.cloth_sphere(16)
    s = Session(sc)
    g0, it0 = lib.ppf_graph_launches(), _graph_stats(lib)
    newton = 0
    for _ in range(6):
        assert s.step().success()
        newton += s.stats().newton_iters
    assert lib.ppf_graph_launches() - g0 == newton
    assert (_graph_stats(lib) == it0).all()
    # a constraint update re-captures; the next step still matches the oracle
    lib.update_constraint(sc.constraint)
    o = OracleSession(sc)
    g1 = lib.ppf_graph_launches()
    rg, ro = s.step(), o.step()
    assert rg.success() and ro.success()
    assert lib.ppf_graph_launches() - g1 == s.stats().newton_iters
    xg, xo = s.positions(), o.positions()[0]
    assert np.abs(xg - xo).max() <= 1e-5 * np.abs(xo).max()


def test_newton_iteration_replays_as_one_graph(lib):
    from oracle.binding import OracleSession

    sc, _ = scenes.cloth_sphere(16)
    s = Session(sc)
    a = _graph_stats(lib)
    newton = 0
    for _ in range(6):
        assert s.step().success()
        newton += s.stats().newton_iters
    d = _graph_stats(lib) - a
    # every iteration ran in the graph path: at most once directly under a
    # new key, once captured, the rest replayed (a scene of the same sizes in
    # the same buffers as the last one captured replays its graph at once)
    assert d[0] + d[2] == newton, d
    assert d[0] <= 1 and d[1] <= 1 and d[3] == 0, d
    # a constraint update rewrites the device arrays in place: the captured
    # graph stays valid, and its next step matches the oracle's
    lib.update_constraint(sc.constraint)
    o = OracleSession(sc)
    b = _graph_stats(lib)
    rg, ro = s.step(), o.step()
    assert rg.success() and ro.success()
    d = _graph_stats(lib) - b
    assert d[0] == 0 and d[1] == 0 and d[2] == s.stats().newton_iters, d
    xg, xo = s.positions(), o.positions()[0]
    assert np.abs(xg - xo).max() <= 1e-5 * np.abs(xo).max()


def test_graph_and_sized_assembly_agree(lib):
    """The same 8 steps with the iteration graph on and off: the two differ
    only by the order of the float atomics in the assembly."""
    runs = []
    for on in (1, 0):
        lib.ppf_set_iteration_graph(on)
        sc, _ = scenes.cloth_sphere(16)
        s = Session(sc)
        for _ in range(8):
            assert s.step().success()
        runs.append(s.positions())
    xg, xs = runs
    assert np.abs(xg - xs).max() <= 1e-5 * np.abs(xs).max()


@pytest.mark.parametrize("caps", [(8, 0), (0, 16), (8, 16)])
def test_overrun_iteration_is_repeated(lib, caps):
    """two_sheets after three oracle steps has point-face, point-edge,
    point-point and edge-edge pairs; with the pair lists capped at 8 entries
    and / or the contact blocks at 16, the first iteration overruns, is
    repeated with grown capacities, and the step matches the oracle's."""
    from oracle.binding import OracleSession

    sc, _ = step_scenes.two_sheets()
    orc = OracleSession(sc)
    for _ in range(3):
        assert orc.step().success()
    curr, prev = orc.positions()
    sc.set_positions(curr, prev)
    sc.param.contents.time = orc.time
    s = Session(sc)
    o = OracleSession(sc)
    lib.ppf_debug_set_contact_capacity(*caps)
    a = _graph_stats(lib)
    rg, ro = s.step(), o.step()
    assert rg.success() and ro.success(), (rg.as_dict(), ro.as_dict())
    d = _graph_stats(lib) - a
    assert d[3] >= 1, d
    # a repeated iteration ran twice (or more) and counts once
    assert d[0] + d[2] == s.stats().newton_iters + d[3], d
    xg, xo = s.positions(), o.positions()[0]
    assert np.abs(xg - xo).max() <= 1e-5 * np.abs(xo).max()
