"""The line-search stage of every Newton iteration runs as one replayed CUDA
graph (ppf_graph_launches): one replay per Newton iteration, re-captured
after update_constraint, and the steps it takes are the oracle's (one step
from an identical state within 1e-5 relative)."""
import ctypes as C

import numpy as np
import pytest

from ppf_gb300 import scenes
from ppf_gb300.session import Session

pytestmark = pytest.mark.gpu


def test_line_search_stage_replays_as_a_graph(oracle_lib, product_lib):
    from oracle.binding import OracleSession

    lib = product_lib
    lib.ppf_graph_launches.restype = C.c_ulonglong
    sc, _ = scenes.cloth_sphere(16)
    s = Session(sc)
    g0 = lib.ppf_graph_launches()
    newton = 0
    for _ in range(6):
        assert s.step().success()
        newton += s.stats().newton_iters
    assert lib.ppf_graph_launches() - g0 == newton
    # a constraint update re-captures; the next step still matches the oracle
    lib.update_constraint(sc.constraint)
    o = OracleSession(sc)
    g1 = lib.ppf_graph_launches()
    rg, ro = s.step(), o.step()
    assert rg.success() and ro.success()
    assert lib.ppf_graph_launches() - g1 == s.stats().newton_iters
    xg, xo = s.positions(), o.positions()[0]
    assert np.abs(xg - xo).max() <= 1e-5 * np.abs(xo).max()
