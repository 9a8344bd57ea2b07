"""Batched PCG over many independent systems (ppf_batch_pcg).

CPU: the packed both-triangle layout is the system's operator.
GPU: one launch over many systems gives each system the bits it gets alone;
every system is solved to the tolerance, in the iterations a float64
restatement of the same PCG takes; captured uneven drops all converge.
"""
import numpy as np
import pytest

import learned_cases
from oracle import fsai as OF


def _dense_from_packed(packed, s):
    row_off, off, col, val, _ = packed
    lo, hi = int(row_off[s]), int(row_off[s + 1])
    n = hi - lo
    A = np.zeros((3 * n, 3 * n))
    for i in range(lo, hi):
        for k in range(int(off[i]), int(off[i + 1])):
            j = int(col[k]) - lo
            A[3 * (i - lo):3 * (i - lo) + 3, 3 * j:3 * j + 3] = \
                val[9 * k:9 * k + 9].reshape(3, 3).T
    return A


def _samples(seeds, n=300):
    out = []
    for k in seeds:
        s = learned_cases.synthetic(n=n, seed=k)
        A = OF.dense_operator(learned_cases.graph(s))
        free = np.repeat(s["dof"] == 0, 3)
        b = np.random.default_rng(k).normal(size=3 * n) * free
        s["force"] = b.astype(np.float32)
        s["A"] = A
        out.append(s)
    return out


def _pcg_iters(A, b, tol=1e-3, maxit=10000):
    """The PCG of the kernel in float64: x0 = 0, block-Jacobi, relative L1
    residual checked at iterations 1, 5, 9, ... and every iteration once
    below 8 tol."""
    n = len(b) // 3
    Pinv = np.zeros_like(A)
    for i in range(n):
        Pinv[3 * i:3 * i + 3, 3 * i:3 * i + 3] = np.linalg.inv(A[3 * i:3 * i + 3, 3 * i:3 * i + 3])
    x = np.zeros_like(b)
    r = b.copy()
    z = Pinv @ r
    p = z.copy()
    rz = r @ z
    err0 = np.abs(r).sum()
    stride, nxt = 4, 1
    for it in range(1, maxit + 1):
        Ap = A @ p
        a = rz / (p @ Ap)
        x += a * p
        r -= a * Ap
        z = Pinv @ r
        rz1 = r @ z
        if it == nxt:
            rr = np.abs(r).sum() / err0
            if rr < tol:
                return it
            if rr < 8 * tol:
                stride = 1
            nxt = it + stride
        p = z + rz1 / rz * p
        rz = rz1
    return maxit


def test_packed_rows_are_the_operator():
    from ppf_gb300 import batch

    samples = _samples([1, 2, 3], n=60)
    packed = batch.pack(samples)
    assert packed[0].tolist() == [0, 60, 120, 180]
    for s, smp in enumerate(samples):
        np.testing.assert_allclose(_dense_from_packed(packed, s), smp["A"], rtol=0, atol=1e-6)
        np.testing.assert_array_equal(packed[4][3 * 60 * s:3 * 60 * (s + 1)], smp["force"])


def test_batch_rejects_invalid_input(product_lib):
    """The batch entry points check their input on the host before any device
    work (so this runs without a GPU): a column that points into another
    system, decreasing row offsets, an unknown preconditioner and a team size
    that is not 1, 2, 4, 8 or 16 are refused, and a refused table leaves the
    library's table as it was."""
    from ppf_gb300 import abi, batch

    packed = batch.pack(_samples([1, 2], n=40))
    row_off, off, col, val, rhs = packed
    bad_col = col.copy()
    bad_col[0] = 50  # row 0 is system 0's; row 50 is system 1's
    with pytest.raises(ValueError):
        batch.solve((row_off, off, bad_col, val, rhs))
    bad_rows = row_off.copy()
    bad_rows[1] = 90  # past the end of the next system
    with pytest.raises(ValueError):
        batch.solve((bad_rows, off, col, val, rhs))
    with pytest.raises(ValueError):
        batch.solve(packed, precond=3)
    assert abi.PRECOND_FSAI != 3
    before = batch.team_ctas().tolist()
    with pytest.raises(ValueError):
        batch.team_ctas([1, 3, 1, 1, 1])
    assert batch.team_ctas().tolist() == before


def test_refine_keeps_the_fastest_whole_batch_table(monkeypatch):
    """The whole-batch refinement (CPU, with the library calls replaced by a
    cost model): it moves one bucket at a time to a faster team size, tries
    only the sizes the per-bucket tuner could run, ignores changes within the
    noise margin, and leaves the library's table at its answer."""
    from ppf_gb300 import batch

    state = {"table": [1, 1, 1, 1, 1], "calls": 0}

    def fake_team_ctas(table=None):
        if table is not None:
            state["table"] = [int(v) for v in table]
        return np.array(state["table"], np.uint32)

    def fake_solve(packed, tol=1e-3, max_iter=10000, **kw):
        t = state["table"]
        state["calls"] += 1
        # bucket 3 is best at 4 CTAs, bucket 4 at 16, bucket 1 indifferent
        # within 0.5 %; bucket 0 and 2 fixed by the tuner's ms
        ms = 30.0 + 3.0 * abs(t[3] - 4) / 4 + (0.0 if t[4] == 16 else 5.0)
        ms += 0.1 if t[1] == 1 else 0.0
        return {"ms": ms}

    monkeypatch.setattr(batch, "team_ctas", fake_team_ctas)
    monkeypatch.setattr(batch, "solve", fake_solve)
    ms = np.full((5, 5), -1.0)
    ms[0, 0] = 1.0
    ms[1, :2] = [2.0, 1.5]
    ms[3, :4] = [9.0, 5.0, 3.0, 2.0]
    ms[4, :] = [9.0, 6.0, 4.0, 3.0, 2.0]
    table, best = batch.refine(None, [1, 2, 1, 8, 16], ms, reps=1)
    assert table.tolist() == [1, 2, 1, 4, 16] and best == 30.0
    assert state["table"] == [1, 2, 1, 4, 16]
    # a start away from the optimum in two buckets
    table, best = batch.refine(None, [1, 2, 1, 1, 2], ms, reps=1)
    assert table.tolist() == [1, 2, 1, 4, 16] and best == 30.0


@pytest.mark.gpu
def test_batch_equals_one_launch_per_system(product_lib):
    from ppf_gb300 import batch

    samples = _samples(range(10, 16))
    packed = batch.pack(samples)
    a = batch.solve(packed)
    b = batch.solve(packed, one_by_one=True)
    assert np.array_equal(a["x"], b["x"])
    assert np.array_equal(a["iters"], b["iters"])
    # a system alone in its own batch
    one = batch.solve(batch.pack(samples[2:3]))
    assert np.array_equal(one["x"], a["x"][600:900]) and one["iters"][0] == a["iters"][2]


@pytest.mark.gpu
def test_cluster_teams_for_large_systems(product_lib):
    """Systems above 2,048 vertices run on clusters of CTAs (partial sums
    through distributed shared memory): a batch mixing them with small ones
    gives every system the bits it gets alone, and solves it."""
    from ppf_gb300 import batch

    samples = _samples([31], n=300) + _samples([32], n=3000) + _samples([33], n=5000)
    packed = batch.pack(samples)
    a = batch.solve(packed)
    b = batch.solve(packed, one_by_one=True)
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["iters"], b["iters"])
    assert np.all(a["state"] == 0)
    base = 0
    for s, smp in enumerate(samples):
        n = int(smp["n"])
        x = a["x"][base:base + n].reshape(-1).astype(np.float64)
        bb = smp["force"].astype(np.float64)
        assert np.abs(bb - smp["A"] @ x).sum() / np.abs(bb).sum() < 2e-3
        base += n


@pytest.mark.gpu
def test_autotuned_team_sizes(product_lib):
    """The autotuner picks a measured team size per size bucket, and a batch
    solved with any table gives every system the bits it gets alone."""
    from ppf_gb300 import batch

    samples = _samples([41], n=300) + _samples([42], n=1500) + _samples([43], n=3000)
    packed = batch.pack(samples)
    default = batch.team_ctas()
    try:
        table, ms = batch.autotune(packed)
        for b in (0, 1, 2):  # the buckets present
            tried = ms[b][ms[b] >= 0]
            assert tried.size >= 1 and table[b] in batch.TEAM_SIZES
            assert ms[b][batch.TEAM_SIZES.index(int(table[b]))] == tried.min()
        for t in (table, np.array([1, 1, 1, 1, 1]), np.array([2, 4, 4, 8, 8])):
            batch.team_ctas(t)
            a = batch.solve(packed)
            b = batch.solve(packed, one_by_one=True)
            assert np.array_equal(a["x"], b["x"]) and np.all(a["state"] == 0)
    finally:
        batch.team_ctas(default)


@pytest.mark.gpu
def test_fsai_batch(product_lib):
    """The batch with each system's FSAI factor (built on the device): every
    system solved, in fewer iterations than with block-Jacobi, with the bits
    one launch per system gives; a hub row keeps its 15 strongest couplings,
    and a cluster-sized system is included."""
    from ppf_gb300 import abi, batch

    samples = _samples(range(50, 54)) + _samples([55], n=3000)
    hub = learned_cases.synthetic(n=200, seed=56, hub=60)
    hub["A"] = OF.dense_operator(learned_cases.graph(hub))
    hub["force"] = (np.random.default_rng(56).normal(size=600) *
                    np.repeat(hub["dof"] == 0, 3)).astype(np.float32)
    samples.append(hub)
    packed = batch.pack(samples)
    bj = batch.solve(packed)
    fs = batch.solve(packed, precond=abi.PRECOND_FSAI)
    one = batch.solve(packed, precond=abi.PRECOND_FSAI, one_by_one=True)
    assert np.array_equal(fs["x"], one["x"]) and np.array_equal(fs["iters"], one["iters"])
    assert np.all(fs["state"] == 0)
    base = 0
    for s, smp in enumerate(samples):
        n = int(smp["n"])
        x = fs["x"][base:base + n].reshape(-1).astype(np.float64)
        b = smp["force"].astype(np.float64)
        assert np.abs(b - smp["A"] @ x).sum() / np.abs(b).sum() < 2e-3, s
        base += n
    # the synthetic systems converge by the first checks either way; the gain
    # shows on the Newton systems the solver assembles
    drops = [batch.capture_drop(p) for p in [(32, 0.2, "sphere", 0.3), (40, 0.25, "box", 0.4),
                                             (24, 0.2, "sphere", 0.2)]]
    dp = batch.pack(drops)
    bj = batch.solve(dp)
    fs = batch.solve(dp, precond=abi.PRECOND_FSAI)
    assert np.all(fs["state"] == 0) and np.all(bj["state"] == 0)
    assert fs["iters"].sum() < 0.8 * bj["iters"].sum(), (fs["iters"], bj["iters"])


@pytest.mark.gpu
def test_batch_solves_every_system(product_lib):
    from ppf_gb300 import batch

    samples = _samples(range(20, 26))
    packed = batch.pack(samples)
    out = batch.solve(packed)
    assert np.all(out["state"] == 0)
    for s, smp in enumerate(samples):
        x = out["x"][300 * s:300 * (s + 1)].reshape(-1).astype(np.float64)
        b = smp["force"].astype(np.float64)
        res = np.abs(b - smp["A"] @ x).sum() / np.abs(b).sum()
        assert res < 2e-3, (s, res)
        it = _pcg_iters(smp["A"], b)
        assert abs(int(out["iters"][s]) - it) <= 4, (s, out["iters"][s], it)


@pytest.mark.gpu
def test_batch_of_captured_uneven_drops(product_lib):
    """Newton systems the solver assembles for a few uneven drops (sphere and
    box colliders, sides 16-40), solved in one launch."""
    from ppf_gb300 import batch

    params = [(16, 0.2, "sphere", 0.2), (24, 0.3, "box", 0.4), (40, 0.25, "sphere", 0.35),
              (20, 0.2, "box", 0.3)]
    samples = [batch.capture_drop(p) for p in params]
    packed = batch.pack(samples)
    out = batch.solve(packed)
    assert np.all(out["state"] == 0), out["state"]
    base = 0
    for s, smp in enumerate(samples):
        n = int(smp["n"])
        x = out["x"][base:base + n].reshape(-1).astype(np.float64)
        A = _dense_from_packed(packed, s)
        b = smp["force"].astype(np.float64).reshape(-1)
        assert np.abs(b - A @ x).sum() / np.abs(b).sum() < 2e-3
        base += n
