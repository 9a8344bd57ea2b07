"""States and comparisons for pinning the oracle's Newton-system assembly,
line searches and intersection check to the reference's own code.

The reference side is oracle/ref_pipeline.cpp: the reference's energy.cu,
strainlimiting.cu and contact.cu compiled as host code. Both sides assemble
the first Newton system of a step at the same state (eval_x = curr, the
oracle's target and dt) before the Dirichlet elimination of main.cu:954-1049,
which is not part of those files. The matrix is compared as the sum of every
stored upper-triangle block per (row, col), so the split between the fixed
pattern, the contact rows and the per-vertex diagonal does not matter.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ppf_gb300 import abi

STEPS = 3  # oracle steps of the two-sheets scene at which systems are compared


def canonical(rows, cols, vals):
    """(keys, blocks): sorted unique row << 32 | col and the summed 3x3 blocks
    (9 floats, column-major), summed in float64."""
    keys = (rows.astype(np.uint64) << np.uint64(32)) | cols.astype(np.uint64)
    uk, inv = np.unique(keys, return_inverse=True)
    out = np.zeros((len(uk), 9), np.float64)
    np.add.at(out, inv, vals.reshape(-1, 9).astype(np.float64))
    return uk, out


def oracle_blocks(sysd, n):
    """Upper blocks of the oracle's system (fixed pattern with the diagonal
    folded in, plus the contact blocks)."""
    f_rows = np.repeat(np.arange(n, dtype=np.uint32), np.diff(sysd["f_off"]))
    d_rows = np.repeat(np.arange(n, dtype=np.uint32), np.diff(sysd["d_off"]))
    rows = np.concatenate([f_rows, d_rows])
    cols = np.concatenate([sysd["f_col"], sysd["d_col"]])
    vals = np.concatenate([sysd["f_val"], sysd["d_val"]])
    return canonical(rows, cols, vals)


def reference_blocks(lib):
    k = lib.refpipe_blocks(None, None, None)
    rows = np.zeros(k, np.uint32)
    cols = np.zeros(k, np.uint32)
    vals = np.zeros(9 * k, np.float32)
    lib.refpipe_blocks(rows, cols, vals)
    return canonical(rows, cols, vals)


def oracle_param(o):
    prm = abi.ParamSet()
    o.lib.oracle_param(C.byref(prm))
    return prm


def oracle_first_system(o):
    """The oracle's first Newton system of its next step, without Dirichlet
    elimination: (curr, prev, param, target, dt, keys, blocks, force)."""
    curr, prev = o.positions()
    prm = oracle_param(o)
    target = np.zeros(3 * o.n, np.float32)
    dt = o.lib.oracle_assemble_first(0, target)
    sysd = o.system()
    keys, blocks = oracle_blocks(sysd, o.n)
    return (curr.reshape(-1).copy(), prev.reshape(-1).copy(), prm, target, float(dt), keys,
            blocks, sysd["force"].reshape(-1).copy())


def dataset_positions(sc):
    """(curr, prev) of a built scene in the DataSet's vertex order (which puts
    a solid's interior vertices last), flattened."""
    curr, prev = sc.positions()
    order = sc.array("vertex_order")
    c = np.empty_like(curr)
    p = np.empty_like(prev)
    c[order] = curr
    p[order] = prev
    return c.reshape(-1).copy(), p.reshape(-1).copy()


def step_target(sc, curr, prev):
    """The inertial target of a step from (curr, prev) as the library and the
    reference compute it in float32 (main.cu:491-511): x + (x - x_prev)
    dt / dt_prev + dt^2 g for free vertices (the scenes used here have no
    pins)."""
    p = sc.param.contents
    f32 = np.float32
    dt = f32(p.dt) * f32(p.playback)
    tr = dt / f32(p.prev_dt)
    h2 = dt * dt
    g = np.array([p.gravity.v[0], p.gravity.v[1], p.gravity.v[2]], f32)
    x1 = curr.reshape(-1, 3).astype(f32)
    x0 = prev.reshape(-1, 3).astype(f32)
    y = (x1 - x0) * tr + h2 * g
    return (x1 + y).reshape(-1).astype(f32)


def reference_first_system(lib, curr, prev, prm, target, dt):
    lib.refpipe_state(curr, prev, C.byref(prm))
    count = lib.refpipe_assemble(curr, target, dt)
    force = np.zeros(len(curr), np.float32)
    lib.refpipe_force(force)
    keys, blocks = reference_blocks(lib)
    return keys, blocks, force, int(count)


def block_scale(keys, blocks, n):
    """Per block, the larger of its two diagonal blocks' largest entries."""
    rows = (keys >> np.uint64(32)).astype(np.int64)
    cols = (keys & np.uint64(0xFFFFFFFF)).astype(np.int64)
    diag = np.zeros(n)
    on = rows == cols
    diag[rows[on]] = np.abs(blocks[on]).max(axis=1)
    return np.maximum(diag[rows], diag[cols])


def compare_systems(n, ref, orc, tol=1e-5):
    """Asserts the same block pattern, every block within tol of its diagonal
    scale, and the force within tol of its largest entry."""
    rk, rb, rf = ref
    ok, ob, of = orc
    only_ref = np.setdiff1d(rk, ok)
    only_orc = np.setdiff1d(ok, rk)
    assert len(only_ref) == 0 and len(only_orc) == 0, (
        f"block patterns differ: {len(only_ref)} only in the reference, "
        f"{len(only_orc)} only in the oracle")
    scale = block_scale(rk, rb, n)
    err = np.abs(rb - ob).max(axis=1)
    worst = int(np.argmax(err / scale))
    assert np.all(err <= tol * scale), (
        f"block ({int(rk[worst] >> np.uint64(32))}, {int(rk[worst] & np.uint64(0xFFFFFFFF))}): "
        f"|diff| {err[worst]:.3e} vs diagonal scale {scale[worst]:.3e}")
    fs = np.abs(rf).max()
    assert np.all(np.abs(rf.astype(np.float64) - of) <= tol * fs), (
        f"force: max |diff| {np.abs(rf.astype(np.float64) - of).max():.3e} vs {fs:.3e}")


def line_search_cases(x0, dx):
    """End states x1 for the line searches from x0: the oracle's Newton
    direction, sheet B dropped through sheet A, the small triangle raised
    into sheet A, and a 3 % stretch along x (strain limit)."""
    x = x0.reshape(-1, 3)
    cases = {"newton": (x0 - dx.reshape(-1)).astype(np.float32)}
    down = x.copy()
    down[144:287, 1] -= 3e-3
    cases["sheet_b_down"] = down.reshape(-1)
    up = x.copy()
    up[-3:, 1] += 2e-3
    cases["triangle_up"] = up.reshape(-1)
    stretch = x.copy()
    stretch[:, 0] *= 1.03
    cases["stretch"] = stretch.reshape(-1)
    return cases


def intersection_cases(x0):
    """States for the intersection check: the start state (free) and sheet B
    tilted through sheet A (intersecting)."""
    x = x0.reshape(-1, 3)
    tilt = x.copy()
    xb = tilt[144:287, 0]
    tilt[144:287, 1] -= 0.05 * (xb - xb.mean())
    return {"start": x0, "tilted": tilt.reshape(-1).astype(np.float32)}
