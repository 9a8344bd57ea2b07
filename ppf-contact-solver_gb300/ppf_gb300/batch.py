"""Batched PCG over many independent Newton systems (ppf_batch_pcg).

A batch of uneven scenes (the reference runs one scene per process) gives
many small Newton systems at a time. ppf_batch_pcg solves all of them with the
reference's block-Jacobi PCG (or each system's FSAI factor) in one launch per
team size, one team (a CTA or a thread-block cluster) per system, each to its
own tolerance and iteration count. This module packs the systems the solver
itself assembles (ppf_debug_newton_system) into that launch's layout and
drives it.

Usage (on a GPU):
    python -m ppf_gb300.batch bench [--count 256]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time

import numpy as np

from . import abi, learned, scenes
from ._lib import f32p, f32p_opt, product, u32p
from .session import Session

_declared = set()


def _declare(lib):
    if id(lib) in _declared:
        return
    lib.ppf_batch_pcg.restype = C.c_int
    lib.ppf_batch_pcg.argtypes = [C.c_uint, u32p, u32p, u32p, f32p, f32p, C.c_float, C.c_uint,
                                  C.c_int, C.c_int, f32p_opt, np.ctypeslib.ndpointer(np.uint32, flags="C"),
                                  f32p_opt, np.ctypeslib.ndpointer(np.int32, flags="C"),
                                  C.POINTER(C.c_float)]
    lib.ppf_batch_team_ctas.restype = C.c_int
    lib.ppf_batch_team_ctas.argtypes = [u32p, C.c_int]
    lib.ppf_batch_autotune.restype = C.c_int
    lib.ppf_batch_autotune.argtypes = [C.c_uint, u32p, u32p, u32p, f32p, f32p, C.c_float,
                                       C.c_uint, u32p, f32p]
    _declared.add(id(lib))


BUCKETS = ("<=1024 rows", "<=2048", "<=4096", "<=8192", ">8192")
TEAM_SIZES = (1, 2, 4, 8, 16)


def team_ctas(table=None):
    """The team size per size bucket (reads it; with `table`, sets it)."""
    lib = product()
    _declare(lib)
    t = np.zeros(5, np.uint32) if table is None else np.ascontiguousarray(table, np.uint32)
    if lib.ppf_batch_team_ctas(t, 0 if table is None else 1) != 0:
        raise ValueError("invalid team sizes")
    return t


def autotune(packed, tol: float = 1e-3, max_iter: int = 10000):
    """Measures each team size on all of the batch's systems of a size bucket
    at once and keeps the fastest per bucket; returns (table, ms[5, 5])."""
    lib = product()
    _declare(lib)
    row_off, off, col, val, rhs = packed
    table = np.zeros(5, np.uint32)
    ms = np.full(25, -1.0, np.float32)
    if lib.ppf_batch_autotune(len(row_off) - 1, row_off, off, col, val, rhs, tol, max_iter,
                              table, ms) != 0:
        raise ValueError("the library rejected the batch")
    return table, ms.reshape(5, 5)


def refine(packed, table, ms, tol: float = 1e-3, max_iter: int = 10000, reps: int = 3,
           rounds: int = 2, margin: float = 0.01):
    """Whole-batch refinement of a per-bucket table (autotune's).

    autotune times each bucket's systems alone. In a batch all buckets share
    the GPU, and a smaller team in one bucket can leave room for the others.
    Coordinate descent: each present bucket in turn tries the team sizes
    autotune could run (ms >= 0), timing the whole batch (best of `reps`),
    and keeps a change that saves more than `margin`; at most `rounds`
    sweeps. Sets the library's table to the result and returns
    (table, batch ms)."""
    ms = np.asarray(ms).reshape(5, 5)

    def cost(t):
        team_ctas(t)
        return min(solve(packed, tol, max_iter)["ms"] for _ in range(reps))

    best_t = [int(v) for v in table]
    best = cost(best_t)
    seen = {tuple(best_t): best}
    for _ in range(rounds):
        improved = False
        for b in range(5):
            if not (ms[b] >= 0).any():
                continue  # no system in this bucket
            for c, size in enumerate(TEAM_SIZES):
                if ms[b, c] < 0 or size == best_t[b]:
                    continue
                t = list(best_t)
                t[b] = size
                if tuple(t) in seen:
                    continue
                m = seen[tuple(t)] = cost(t)
                if m < best * (1.0 - margin):
                    best, best_t, improved = m, t, True
        if not improved:
            break
    team_ctas(best_t)
    return np.array(best_t, np.uint32), best


def full_rows(sample: dict):
    """Both-triangle block rows (off, col, val) of a captured Newton system:
    every upper block (r, c) of the fixed pattern and the contact blocks, and
    its transpose at (c, r) off the diagonal."""
    n = int(sample["n"])
    parts = []
    for off, col, val in ((sample["f_off"], sample["f_col"], sample["f_val"]),
                          (sample["d_off"], sample["d_col"], sample["d_val"])):
        off = np.asarray(off, np.int64)
        m = int(off[-1])
        if m == 0:
            continue
        row = np.repeat(np.arange(n), np.diff(off))
        col = np.asarray(col, np.int64)[:m]
        blk = np.asarray(val, np.float32)[:9 * m].reshape(m, 9)
        parts.append((row, col, blk))
        odd = row != col
        tr = blk[odd].reshape(-1, 3, 3).transpose(0, 2, 1).reshape(-1, 9)
        parts.append((col[odd], row[odd], tr))
    rows = np.concatenate([p[0] for p in parts])
    cols = np.concatenate([p[1] for p in parts])
    vals = np.concatenate([p[2] for p in parts])
    order = np.lexsort((cols, rows))
    off = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).astype(np.uint32)
    return off, cols[order].astype(np.uint32), np.ascontiguousarray(vals[order].reshape(-1))


def pack(samples):
    """The launch's layout of a list of captured systems: (row_off, off, col,
    val, rhs) over all systems, columns as global rows."""
    row_off, offs, cols, vals, rhs = [0], [], [], [], []
    base_blocks = 0
    for s in samples:
        off, col, val = full_rows(s)
        base = row_off[-1]
        offs.append(off[:-1].astype(np.int64) + base_blocks)
        cols.append(col.astype(np.int64) + base)
        vals.append(val)
        rhs.append(np.asarray(s["force"], np.float32).reshape(-1))
        base_blocks += int(off[-1])
        row_off.append(base + int(s["n"]))
    off = np.concatenate(offs + [np.array([base_blocks])]).astype(np.uint32)
    return (np.array(row_off, np.uint32), off, np.concatenate(cols).astype(np.uint32),
            np.concatenate(vals).astype(np.float32), np.concatenate(rhs).astype(np.float32))


def solve(packed, tol: float = 1e-3, max_iter: int = 10000, one_by_one: bool = False,
          precond: int = abi.PRECOND_BLOCK_JACOBI) -> dict:
    """Solves every packed system (block-Jacobi, or abi.PRECOND_FSAI); returns
    x (rows x 3), and per system the iterations, relative L1 residual and
    state, and the device time (the operator's SELL-32 copy and the FSAI
    factor build included)."""
    lib = product()
    _declare(lib)
    row_off, off, col, val, rhs = packed
    ns = len(row_off) - 1
    rows = int(row_off[-1])
    x = np.zeros(3 * rows, np.float32)
    it = np.zeros(ns, np.uint32)
    res = np.zeros(ns, np.float32)
    st = np.zeros(ns, np.int32)
    ms = C.c_float()
    rc = lib.ppf_batch_pcg(ns, row_off, off, col, val, rhs, tol, max_iter, int(precond),
                           int(one_by_one), x, it, res, st, C.byref(ms))
    if rc != 0:
        raise ValueError("the library rejected the batch")
    return {"x": x.reshape(-1, 3), "iters": it, "resid": res, "state": st, "ms": ms.value}


def capture_drop(params, extra_steps: int = 3) -> dict:
    """Steps one uneven drop with block-Jacobi until the sheet has fallen onto
    its collider (free-fall time of its height, plus a few steps) and
    captures that step's Newton system."""
    side, height, collider, size = params
    sc, _ = scenes.cloth_drop(side, height, collider, size)
    sess = Session(sc)
    sess.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
    steps = int(math.ceil(math.sqrt(2.0 * height / 9.8) / 0.01)) + extra_steps
    for _ in range(steps):
        if not sess.step(fetch=False).success():
            break
    out = learned.capture_system(sc.vertex_count)
    del sess, sc
    return out


def run_bench(count: int = 256, seed: int = 0, reps: int = 3) -> dict:
    """Captures the uneven drops' Newton systems, autotunes the team sizes
    (per bucket, then refined on the whole batch) and times the batch
    against one launch per system; returns the figures.
    Leaves the library's team-size table as it found it."""
    a = argparse.Namespace(count=count, seed=seed, reps=reps)
    t0 = time.time()
    params = scenes.uneven_drops(a.count, a.seed)
    samples = [capture_drop(p) for p in params]
    capture_s = time.time() - t0
    packed = pack(samples)
    default_table = team_ctas()
    solve(packed)  # warm-up
    default_ms = min(solve(packed)["ms"] for _ in range(a.reps))
    bucket_table, tune_ms = autotune(packed)
    table, _ = refine(packed, bucket_table, tune_ms)
    batched = min((solve(packed) for _ in range(a.reps)), key=lambda r: r["ms"])
    single = min((solve(packed, one_by_one=True) for _ in range(a.reps)), key=lambda r: r["ms"])
    same = bool(np.array_equal(batched["x"], single["x"]) and
                np.array_equal(batched["iters"], single["iters"]))
    fsai = min((solve(packed, precond=abi.PRECOND_FSAI) for _ in range(a.reps)),
               key=lambda r: r["ms"])
    fit = np.sort(fsai["iters"])
    # the largest system alone: the floor of a batch whose systems each run
    # on one CTA
    big = int(np.argmax([int(packed[1][packed[0][k + 1]] - packed[1][packed[0][k]])
                         for k in range(a.count)]))
    alone = min(solve(pack(samples[big:big + 1]))["ms"] for _ in range(a.reps))
    it = np.sort(batched["iters"])
    verts = [int(s["n"]) for s in samples]
    out = {
        "workload": f"{a.count} uneven cloth drops (sides 16-96 log-uniform, heights 0.2-1.0 m, "
                    "sphere or box colliders; seeded), the Newton system of the step where "
                    "each sheet meets its collider",
        "systems": a.count, "vertices_total": int(sum(verts)),
        "vertices_min_max": [min(verts), max(verts)], "blocks": int(packed[1][-1]),
        "batched_ms": round(batched["ms"], 3), "one_launch_per_system_ms": round(single["ms"], 3),
        "team_ctas_default": [int(v) for v in default_table], "batched_ms_default_teams":
            round(default_ms, 3), "team_ctas_per_bucket": [int(v) for v in bucket_table],
        "team_ctas_autotuned": [int(v) for v in table],
        "autotune_ms": {BUCKETS[b]: {str(TEAM_SIZES[c]): round(float(tune_ms[b, c]), 3)
                                     for c in range(5) if tune_ms[b, c] >= 0}
                        for b in range(5) if (tune_ms[b] >= 0).any()},
        "speedup": round(single["ms"] / batched["ms"], 2),
        "largest_system_alone_ms": round(alone, 3),
        "largest_system": {"vertices": int(samples[big]["n"]),
                           "pcg_iters": int(batched["iters"][big])},
        "systems_per_s": round(a.count / (batched["ms"] / 1e3), 1),
        "pcg_iters_median": int(it[len(it) // 2]), "pcg_iters_p90": int(it[int(0.9 * len(it))]),
        "pcg_iters_max": int(it[-1]), "converged": int((batched["state"] == 0).sum()),
        "batched_equals_one_by_one": same, "capture_s": round(capture_s, 1),
        "fsai": {"batched_ms": round(fsai["ms"], 3),
                 "speedup_over_block_jacobi": round(batched["ms"] / fsai["ms"], 2),
                 "pcg_iters_median": int(fit[len(fit) // 2]),
                 "pcg_iters_p90": int(fit[int(0.9 * len(fit))]),
                 "converged": int((fsai["state"] == 0).sum())},
    }
    team_ctas(default_table)
    return out


def bench_main(argv=None):
    ap = argparse.ArgumentParser(description="batched PCG over uneven cloth drops")
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    print(json.dumps(run_bench(a.count, a.seed, a.reps)), flush=True)


if __name__ == "__main__":
    import sys

    if len(sys.argv) < 2 or sys.argv[1] != "bench":
        raise SystemExit("usage: python -m ppf_gb300.batch bench [--count N]")
    bench_main(sys.argv[2:])
