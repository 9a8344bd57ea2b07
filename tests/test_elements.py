"""Element math parity: the formulas the CUDA kernels evaluate against the
reference's own element code.

* against tests/golden/elements.npz, frozen from the reference's sources
  compiled by oracle/Makefile (tests/golden/make_golden.py) -- runs anywhere;
* against that reference build live, where its sources are present.

Bar: equal values (signed zeros aside) on the host that froze the goldens;
a 1e-5 relative band elsewhere, for libm differences between hosts.
"""
from pathlib import Path

import numpy as np
import pytest

import element_cases as ec

GOLDEN = Path(__file__).parent / "golden" / "elements.npz"


def _compare(ref, got, exact):
    bad = []
    for k in sorted(ref):
        x, y = ref[k].astype(np.float64), got[k].astype(np.float64)
        if exact or k in ec.EXACT:
            if not np.array_equal(np.nan_to_num(x), np.nan_to_num(y)):
                bad.append((k, "not equal"))
            continue
        scale = np.maximum(np.abs(x).max(axis=1, keepdims=True), 1e-30)
        rel = (np.abs(x - y) / scale).max()
        if rel > ec.TOL.get(k, 1e-5):
            bad.append((k, rel))
    return bad


def test_golden_covers_every_output():
    g = np.load(GOLDEN)
    assert len(g.files) == 55


def test_element_math_matches_golden(oracle_lib):
    golden = dict(np.load(GOLDEN))
    got = ec.evaluate(oracle_lib, "orc_")
    assert set(golden) == set(got)
    assert _compare(golden, got, exact=False) == []


def test_element_math_equals_reference_build(oracle_lib, ref_lib):
    ref = ec.evaluate(ref_lib, "ref_")
    got = ec.evaluate(oracle_lib, "orc_")
    assert _compare(ref, got, exact=True) == []


def test_ccd_reports_overlapping_start(oracle_lib):
    """A pair that starts inside its offset returns 0 and raises the flag."""
    import ctypes as C

    x0 = np.array([0, 1e-5, 0, -1, 0, -1, 1, 0, -1, 0, 0, 1], np.float32)
    x1 = x0.copy()
    x1[1] = -0.01
    ov = np.zeros(1, np.int32)
    f = oracle_lib.orc_ccd
    f.restype = C.c_float
    f.argtypes = [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float,
                  C.c_float, C.c_float, C.c_float, C.POINTER(C.c_int)]
    t = f(0, ec._ptr(x0), ec._ptr(x1), np.float32(1e-4), np.float32(1e-3),
          np.float32(1.25), np.float32(1e-7), ov.ctypes.data_as(C.POINTER(C.c_int)))
    assert t == 0.0 and ov[0] == 1


def test_invert_spd_matches_inverse(oracle_lib):
    import ctypes as C

    rng = np.random.default_rng(3)
    for _ in range(50):
        a = rng.normal(0, 1, (3, 3))
        a = (a @ a.T + 0.5 * np.eye(3)).astype(np.float32)
        out = np.zeros(9, np.float32)
        ok = np.zeros(1, np.int32)
        oracle_lib.orc_invert_spd(ec._ptr(ec._colmajor(a)), ec._ptr(out),
                                  ok.ctypes.data_as(C.POINTER(C.c_int)))
        inv = out.reshape(3, 3).T
        assert ok[0] == 1
        np.testing.assert_allclose(inv @ a, np.eye(3), atol=2e-4)
