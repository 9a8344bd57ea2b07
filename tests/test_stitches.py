"""Stitches (Constraint::stitch): a spring between two barycentric points
with the reference's rest length (half the weighted contact gap), length cap
and raw stiffness (energy.cu:796-884).

CPU: the builder's stitch list and its 36 slots per stitch over the fixed
pattern; the frozen reference system (tests/golden/ref_stitches.npz) against
the reference's own code where its sources are present.

GPU: the stitched sheets' first Newton system against the reference's
assembly of the same state, block by block; a trajectory in which the
stitches pull the two sheets' facing edges together.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import ref_pipeline_cases as rpc
import step_scenes
from ppf_gb300.session import Session

GOLDEN = Path(__file__).parent / "golden" / "ref_stitches.npz"
f32 = np.float32


def _stitches(sc):
    raw = sc.array("stitch").reshape(-1, 13)
    return raw[:, :6], raw[:, 6:12].view(np.float32), raw[:, 12].view(np.float32)


def test_stitch_builder_tables(product_lib):
    sc, _ = step_scenes.stitched_sheets()
    idx, w, k = _stitches(sc)
    assert len(idx) == 10 and np.all(k > 0)
    assert np.allclose(w[:, :3].sum(1), 1.0) and np.allclose(w[:, 3:].sum(1), 1.0)
    off, col = sc.array("fixed_offset"), sc.array("fixed_index")
    slots = sc.array("stitch_slots").reshape(-1, 36)
    for s_, I in enumerate(idx):
        for a in range(6):
            for b in range(6):
                i, j = int(I[a]), int(I[b])
                if i > j:
                    assert slots[s_, 6 * a + b] == 0xFFFFFFFF
                else:
                    r = col[off[i]:off[i + 1]]
                    pos = np.searchsorted(r, j)
                    assert r[pos] == j and slots[s_, 6 * a + b] == off[i] + pos


def test_stitch_golden_matches_reference_build(ref_pipeline_or_none):
    ref = ref_pipeline_or_none
    if ref is None:
        pytest.skip("reference sources not present")
    g = np.load(GOLDEN)
    sc, _ = step_scenes.stitched_sheets()
    prm = sc.param.contents
    assert ref.refpipe_init(sc.dataset, C.byref(prm))
    curr, prev = rpc.dataset_positions(sc)
    target = rpc.step_target(sc, curr, prev)
    dt = float(f32(prm.dt) * f32(prm.playback))
    keys, blocks, force, count = rpc.reference_first_system(ref, curr, prev, prm, target, dt)
    assert np.array_equal(keys, g["keys"])
    assert np.array_equal(blocks.astype(f32), g["blocks"])
    assert np.array_equal(force, g["force"])


@pytest.mark.gpu
def test_stitch_system_matches_reference(product_lib):
    from oracle.binding import product_system

    g = np.load(GOLDEN)
    sc, _ = step_scenes.stitched_sheets()
    n = sc.vertex_count
    s = Session(sc)
    dx = np.zeros(3 * n, f32)
    it, rr = C.c_uint(), C.c_float()
    assert product_lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr)) == 0
    sysm = product_system(product_lib, n)
    keys, blocks = rpc.oracle_blocks(sysm, n)
    rpc.compare_systems(n, (g["keys"], g["blocks"].astype(np.float64), g["force"]),
                        (keys, blocks, sysm["force"].reshape(-1).astype(np.float64)))
    del s


@pytest.mark.gpu
def test_stitches_pull_the_seam_together(product_lib):
    """30 steps: every step succeeds and the stitched points end closer than
    they started (the 2 mm gap exceeds the stitches' 0.5 mm rest length)."""
    sc, _ = step_scenes.stitched_sheets()
    idx, w, _ = _stitches(sc)
    order = sc.array("vertex_order")
    inv = np.argsort(order)

    def gap(x):
        xd = x[inv]
        p0 = np.einsum("sk,skd->sd", w[:, :3], xd[idx[:, :3]])
        p1 = np.einsum("sk,skd->sd", w[:, 3:], xd[idx[:, 3:]])
        return np.linalg.norm(p0 - p1, axis=1)

    g0 = gap(sc.positions()[0])
    s = Session(sc)
    for k in range(30):
        r = s.step()
        assert r.success(), (k, r.as_dict())
    g1 = gap(s.positions())
    assert np.all(np.isfinite(g1)) and g1.mean() < 0.8 * g0.mean(), (g0.mean(), g1.mean())
