"""Solids (tets) and the singular-value shell models.

CPU: the builder's solid arrays against a numpy restatement of the
reference's construction (scene.rs:1840-1921, builder.rs:232-262, 589-660,
1497-1518, mesh.rs:78-95): the vertex order with interior vertices last, tet
volumes and masses, lumped vertex masses and volumes, the inverse rest
matrices, boundary faces (the unshared tet faces, outward) and element
types; the frozen reference outputs (tests/golden/ref_solids.npz) against
the reference's own code where its sources are present.

GPU: the first Newton system of the solids-and-sheet scene (ARAP tets with
damping, SNHk tets, an StVK sheet, solid-sheet and solid-solid contact)
against the reference's assembly of the same state, block by block; and a
trajectory whose steps all succeed with the solids kept intersection-free.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import ref_pipeline_cases as rpc
import step_scenes
from ppf_gb300.session import Session

GOLDEN = Path(__file__).parent / "golden" / "ref_solids.npz"
f32 = np.float32


@pytest.fixture(scope="module")
def solids_scene(product_lib):
    return step_scenes.solids_and_sheet()


def test_solid_builder_matches_restatement(solids_scene):
    sc, info = solids_scene
    x = sc._rest_positions.astype(f32)
    n = len(x)
    order = sc.array("vertex_order")
    # interior vertices (in a tet, on no face or rod) go last, in added order
    surface = np.zeros(n, bool)
    tets_in = np.concatenate([t + i0 for i0, t, _ in sc._solids])
    in_tet = np.zeros(n, bool)
    in_tet[tets_in.reshape(-1)] = True
    # boundary faces of each solid: tet faces seen once
    bfaces = []
    for i0, t, _ in sc._solids:
        t = t.astype(np.int64) + i0
        cnt = {}
        cand = []
        for a, b, c, d in t:
            for f in ((b, c, d), (a, d, c), (a, b, d), (a, c, b)):
                k = tuple(sorted(f))
                cnt[k] = cnt.get(k, 0) + 1
                cand.append(f)
        bfaces += [f for f in cand if cnt[tuple(sorted(f))] == 1]
    bfaces = np.array(bfaces)
    surface[bfaces.reshape(-1)] = True
    shell_faces = sc.array("face").reshape(-1, 3)
    nf_shell = len(shell_faces) - len(bfaces)
    inv_order = np.argsort(order)
    surface[inv_order[shell_faces[:nf_shell].reshape(-1)]] = True
    interior = in_tet & ~surface
    want = np.concatenate([np.flatnonzero(~interior), np.flatnonzero(interior)])
    assert np.array_equal(inv_order, want)
    # boundary faces follow the shell faces, in tet order, oriented outward
    got_b = inv_order[shell_faces[nf_shell:]]
    assert np.array_equal(got_b, bfaces)
    ft = sc.array("face_type")
    assert np.all(ft[:nf_shell] == 0) and np.all(ft[nf_shell:] == 1)
    # volumes, masses, lumped vertex masses and volumes (float32, in order)
    T = sc.array("tet").reshape(-1, 4)
    xd = x[inv_order]
    e0, e1, e2 = (xd[T[:, k]] - xd[T[:, 0]] for k in (1, 2, 3))
    cr = np.stack([e0[:, 1] * e1[:, 2] - e0[:, 2] * e1[:, 1],
                   e0[:, 2] * e1[:, 0] - e0[:, 0] * e1[:, 2],
                   e0[:, 0] * e1[:, 1] - e0[:, 1] * e1[:, 0]], 1)
    vol = np.abs((cr[:, 0] * e2[:, 0] + cr[:, 1] * e2[:, 1]) + cr[:, 2] * e2[:, 2]) / f32(6.0)
    assert np.array_equal(sc.array("tet_volume"), vol.astype(f32))
    dens = np.concatenate([np.full(len(t), f32(m.density)) for _, t, m in sc._solids])
    assert np.array_equal(sc.array("tet_mass"), dens * vol.astype(f32))
    vv = np.zeros(n, f32)
    for i, t in enumerate(T):
        for k in t:
            vv[k] += sc.array("tet_volume")[i] / f32(4.0)
    assert np.array_equal(sc.array("vertex_volume"), vv)
    # inverse rest matrices: [x1-x0, x2-x0, x3-x0]^-1, column-major
    inv = sc.array("inv_rest3x3").reshape(-1, 3, 3).transpose(0, 2, 1)
    D = np.stack([e0, e1, e2], 2).astype(np.float64)
    assert np.allclose(inv, np.linalg.inv(D), rtol=1e-5, atol=1e-5 * np.abs(inv).max())
    # hinges next to a boundary face are marked (they carry no bending)
    assert np.count_nonzero(sc.array("hinge_type")) > 0


def test_solid_golden_matches_reference_build(ref_pipeline_or_none):
    ref = ref_pipeline_or_none
    if ref is None:
        pytest.skip("reference sources not present")
    g = np.load(GOLDEN)
    sc, info = step_scenes.solids_and_sheet()
    prm = sc.param.contents
    assert ref.refpipe_init(sc.dataset, C.byref(prm))
    curr, prev = rpc.dataset_positions(sc)
    target = rpc.step_target(sc, curr, prev)
    assert np.array_equal(target, g["target"])
    dt = float(f32(prm.dt) * f32(prm.playback))
    keys, blocks, force, count = rpc.reference_first_system(ref, curr, prev, prm, target, dt)
    assert np.array_equal(keys, g["keys"]) and count == int(g["contacts"])
    assert np.array_equal(blocks.astype(f32), g["blocks"])
    assert np.array_equal(force, g["force"])


@pytest.mark.gpu
def test_solid_system_matches_reference(product_lib):
    """Every block and force entry of the product's first Newton system of
    the solids-and-sheet scene within 1e-5 of the reference's, on an
    identical block pattern."""
    from oracle.binding import product_system

    g = np.load(GOLDEN)
    sc, info = step_scenes.solids_and_sheet()
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
def test_solid_trajectory(product_lib):
    """40 steps: every step succeeds (each ends intersection-free by the
    library's own check), positions stay finite and above the floor, and
    the ARAP block keeps its volume within 5 %."""
    sc, info = step_scenes.solids_and_sheet()
    T = sc.array("tet").reshape(-1, 4)
    order = sc.array("vertex_order")
    inv_order = np.argsort(order)
    vol0 = sc.array("tet_volume").sum()
    s = Session(sc)
    for k in range(40):
        r = s.step()
        assert r.success(), (k, r.as_dict())
        x = s.positions()
        assert np.all(np.isfinite(x))
    xd = x[inv_order]
    e0, e1, e2 = (xd[T[:, k]] - xd[T[:, 0]] for k in (1, 2, 3))
    vol = np.abs(np.einsum("ij,ij->i", np.cross(e0, e1), e2)).sum() / 6.0
    assert abs(vol / vol0 - 1.0) < 0.05, vol / vol0
    assert x[:, 1].min() >= 0.3 - 1e-6
