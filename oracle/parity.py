"""Parity checks of the product's Newton systems against the oracle's
(TEST INFRASTRUCTURE: used by tests/ and by bench.py's CPU-baseline leg).

Contact pair sets are decided by the same float32 rule on both sides
(contact/contact.cu:432-887: a pair is accepted when its squared distance is
below (ghat + offset)^2), so on one state they are expected to be identical.
The only pairs that may legitimately differ are those whose distance lies
within 1e-6 * ghat of the threshold, where a last-bit difference in the
positions can flip the test. `compare_pair_sets` lists every pair of either
set in that band (distances in float64 from the float32 positions) and
reports whether the sets are equal outside the list.
"""
from __future__ import annotations

import numpy as np

BAND = 1e-6  # relative to ghat


def _rows(a, width):
    a = np.asarray(a, np.int64).reshape(-1, width)
    return a


def _pt_tri(p, a, b, c):
    """Distance from p to the plane point of triangle abc that the
    barycentric solve gives (pairs are accepted in the interior only)."""
    e0, e1, w = b - a, c - a, p - a
    d00 = (e0 * e0).sum(1)
    d01 = (e0 * e1).sum(1)
    d11 = (e1 * e1).sum(1)
    d20 = (w * e0).sum(1)
    d21 = (w * e1).sum(1)
    den = d00 * d11 - d01 * d01
    v = (d11 * d20 - d01 * d21) / den
    u = (d00 * d21 - d01 * d20) / den
    q = a + v[:, None] * e0 + u[:, None] * e1
    return np.linalg.norm(p - q, axis=1)


def _pt_seg(p, a, b):
    e = b - a
    t = ((p - a) * e).sum(1) / (e * e).sum(1)
    return np.linalg.norm(p - (a + t[:, None] * e), axis=1)


def _seg_seg(p0, p1, q0, q1):
    u, v, w = p1 - p0, q1 - q0, p0 - q0
    a, b, c = (u * u).sum(1), (u * v).sum(1), (v * v).sum(1)
    d, e = (u * w).sum(1), (v * w).sum(1)
    den = a * c - b * b
    s = (b * e - c * d) / den
    t = (a * e - b * d) / den
    return np.linalg.norm((p0 + s[:, None] * u) - (q0 + t[:, None] * v), axis=1)


def pair_distances(kind: str, pairs, x, face, edge):
    """Distance of each pair (rows of the product's / oracle's pair lists)
    at positions x, in float64."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    face = np.asarray(face, np.int64).reshape(-1, 3)
    edge = np.asarray(edge, np.int64).reshape(-1, 2)
    if len(pairs) == 0:
        return np.zeros(0)
    if kind == "pf":
        f = face[pairs[:, 1]]
        return _pt_tri(x[pairs[:, 0]], x[f[:, 0]], x[f[:, 1]], x[f[:, 2]])
    if kind == "pe":
        e = edge[pairs[:, 1]]
        return _pt_seg(x[pairs[:, 0]], x[e[:, 0]], x[e[:, 1]])
    if kind == "pp":
        return np.linalg.norm(x[pairs[:, 0]] - x[pairs[:, 1]], axis=1)
    if kind == "ee":
        a, b = edge[pairs[:, 0]], edge[pairs[:, 1]]
        return _seg_seg(x[a[:, 0]], x[a[:, 1]], x[b[:, 0]], x[b[:, 1]])
    raise ValueError(kind)


WIDTH = {"pf": 2, "pe": 3, "pp": 3, "ee": 2}


def compare_pair_sets(sys_a, sys_b, x, face, edge, ghat: float):
    """Pair sets of two Newton systems (dicts with pf/pe/pp/ee rows) at
    positions x. Returns a dict with, per kind, the counts, the pairs listed
    as within BAND * ghat of the threshold, and whether the two sets agree
    outside that list (identity of (vertex/edge, element) and of the
    multiplicity/friction word where the kind carries one)."""
    out = {"band": f"|d - ghat| <= {BAND:g} * ghat", "ghat": ghat, "kinds": {},
           "equal_outside_listed": True, "listed": 0, "pairs": 0}
    for k, w in WIDTH.items():
        a = {tuple(r) for r in _rows(sys_a[k], w).tolist()}
        b = {tuple(r) for r in _rows(sys_b[k], w).tolist()}
        union = np.array(sorted(a | b), np.int64).reshape(-1, w)
        d = pair_distances(k, union[:, :2], x, face, edge)
        near = np.abs(d - ghat) <= BAND * ghat
        listed = {tuple(r) for r in union[near].tolist()}
        diff = (a ^ b) - listed
        out["kinds"][k] = {"a": len(a), "b": len(b), "listed": len(listed),
                           "differ_outside_listed": len(diff),
                           "listed_pairs": sorted(listed)[:32]}
        out["listed"] += len(listed)
        out["pairs"] += len(a)
        if diff:
            out["equal_outside_listed"] = False
    return out


def apply_system(sysm, v):
    """y = A v in float64 for a kept system (fixed upper pattern with the
    per-vertex diagonal folded in, plus the contact blocks), each upper block
    applied with its transpose below the diagonal. Blocks are column-major."""
    v = np.asarray(v, np.float64).reshape(-1, 3)
    n = len(v)
    y = np.zeros((n, 3))
    for off, col, val in ((sysm["f_off"], sysm["f_col"], sysm["f_val"]),
                          (sysm["d_off"], sysm["d_col"], sysm["d_val"])):
        rows = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
        cols = col.astype(np.int64)
        B = val.astype(np.float64).reshape(-1, 3, 3).transpose(0, 2, 1)  # row-major
        np.add.at(y, rows, np.einsum("kij,kj->ki", B, v[cols]))
        lower = rows != cols
        np.add.at(y, cols[lower], np.einsum("kji,kj->ki", B[lower], v[rows[lower]]))
    return y.reshape(-1)


def dyn_blocks(sysm):
    """Contact blocks as sorted (row, col) keys and their values."""
    off = sysm["d_off"].astype(np.int64)
    n = len(off) - 1
    rows = np.repeat(np.arange(n), np.diff(off))
    cols = sysm["d_col"].astype(np.int64)
    order = np.lexsort((cols, rows))
    keys = np.stack([rows[order], cols[order]], 1) if len(order) else np.zeros((0, 2), np.int64)
    vals = sysm["d_val"][order] if len(order) else np.zeros((0, 9), np.float32)
    return keys, vals


def compare_systems(sg, so, x, face, edge, ghat: float):
    """Product system sg against oracle system so on the same state: pair
    sets (listed band), fixed and contact blocks and force relative to their
    scales. Returns a dict of the measured differences."""
    pairs = compare_pair_sets(sg, so, x, face, edge, ghat)
    res = {"pairs": pairs}
    res["fixed_pattern_equal"] = bool(np.array_equal(sg["f_off"], so["f_off"]) and
                                      np.array_equal(sg["f_col"], so["f_col"]))
    scale = float(np.abs(so["f_val"]).max())
    if res["fixed_pattern_equal"]:
        res["fixed_max_err"] = float(np.abs(sg["f_val"] - so["f_val"]).max()) / scale
    kg, vg = dyn_blocks(sg)
    ko, vo = dyn_blocks(so)
    res["contact_blocks"] = int(len(ko))
    res["contact_pattern_equal"] = bool(np.array_equal(kg, ko))
    if res["contact_pattern_equal"] and len(ko):
        res["contact_max_err"] = float(np.abs(vg - vo).max()) / scale
    fscale = float(np.abs(so["force"]).max())
    res["force_max_err"] = float(np.abs(sg["force"] - so["force"]).max()) / fscale
    res["diag_max_err"] = float(np.abs(sg["diag"] - so["diag"]).max()) / scale
    return res
