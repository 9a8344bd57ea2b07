"""Rods: the builder's rod arrays, the rod element math inside a Newton
system, and the rod strain-limit line search, against the reference.

CPU: the builder's rod props (rest and initial lengths, masses, lumped vertex
masses, rest bend angles from the initial shape, length-weighted vertex
contact parameters, edge and rod-bend slot tables) against a numpy
restatement of scene.rs:1540-1655 and builder.rs:476-870, 1289-1466 in
float32; the frozen reference outputs (tests/golden/ref_rods.npz) against
the reference's own code where its sources are present.

GPU: the first Newton system of the rods-and-sheet scene (rod stretch with
damping, rod bending with lagged damping and bent rest angles, the rod
strain-limit barrier, shell membrane and bending with damping, rod-sheet and
rod-rod contact) against the reference's assembly of the same state, block
by block; the rod strain-limit line search against the reference's; and a
trajectory that keeps every rod within its strain limit.
"""
import ctypes as C
import ctypes.util
from pathlib import Path

import numpy as np
import pytest

import ref_pipeline_cases as rpc
import step_scenes
from ppf_gb300.session import Session

GOLDEN = Path(__file__).parent / "golden" / "ref_rods.npz"
f32 = np.float32
_ACOSF = C.CDLL(ctypes.util.find_library("m")).acosf
_ACOSF.restype = C.c_float
_ACOSF.argtypes = [C.c_float]


def _restate(sc):
    """Rod arrays of the built scene restated from its inputs."""
    E = sc.array("edge").reshape(-1, 2).astype(np.int64)
    F = sc.array("face").reshape(-1, 3).astype(np.int64)
    x = sc._rest_positions.astype(f32)
    nr = sc._rod_count
    n = len(x)
    out = {}
    init = np.array([np.sqrt(np.sum((x[b] - x[a]).astype(f32) ** 2, dtype=f32), dtype=f32)
                     for a, b in E[:nr]], f32)
    mats = sc._rod_mats
    out["edge_initial_length"] = init
    out["edge_length"] = init * np.array([m.length_factor for m in mats], f32)
    out["edge_mass"] = np.array([f32(m.density) for m in mats], f32) * init
    # lumped vertex mass: faces (a third each) first, then rod edges (half)
    fmass = sc.array("face_mass")
    vm = np.zeros(n, f32)
    for i, f in enumerate(F):
        for k in f:
            vm[k] += fmass[i] / f32(3.0)
    for i in range(nr):
        for k in E[i]:
            vm[k] += out["edge_mass"][i] / f32(2.0)
    out["vertex_mass"] = vm
    # rest bend angles
    ve = [[] for _ in range(n)]
    for i, e in enumerate(E):
        for k in e:
            ve[k].append(i)
    vf = [[] for _ in range(n)]
    for i, f in enumerate(F):
        for k in f:
            vf[k].append(i)
    ang = np.full(n, f32(np.pi), f32)
    for j in range(n):
        re = [e for e in ve[j] if e < nr]
        if len(re) != 2 or vf[j]:
            continue
        if not (mats[re[0]].bend_rest_from_geometry or mats[re[1]].bend_rest_from_geometry):
            continue
        o = [E[e][1] if E[e][0] == j else E[e][0] for e in re]
        e0, e1 = (x[o[0]] - x[j]).astype(f32), (x[o[1]] - x[j]).astype(f32)
        n0 = np.sqrt(np.sum(e0 * e0, dtype=f32), dtype=f32)
        n1 = np.sqrt(np.sum(e1 * e1, dtype=f32), dtype=f32)
        c = f32(np.sum(e0 * e1, dtype=f32) / (n0 * n1))
        # f32::acos is the C library's acosf, which the restatement calls too
        ang[j] = _ACOSF(C.c_float(np.clip(c, f32(-1.0), f32(1.0))))
    out["rest_bend_angle"] = ang
    return out, ve, vf


@pytest.fixture(scope="module")
def rods_scene(product_lib):
    sc, info = step_scenes.rods_and_sheet()
    return sc, info


def test_rod_builder_matches_restatement(rods_scene):
    sc, info = rods_scene
    want, ve, vf = _restate(sc)
    for name in ("edge_initial_length", "edge_length", "edge_mass", "rest_bend_angle"):
        got = sc.array(name)[:len(want[name])]
        assert np.array_equal(got, want[name]), (name, np.flatnonzero(got != want[name]))
    vm = sc.array("vertex_mass")
    assert np.array_equal(vm, want["vertex_mass"])
    # every interior rod vertex has a bend stencil in the fixed pattern and
    # slot table; edge slots address each rod edge's blocks
    off, col = sc.array("fixed_offset"), sc.array("fixed_index")
    E = sc.array("edge").reshape(-1, 2)

    def slot(i, j):
        if i > j:
            return 0xFFFFFFFF
        r = col[off[i]:off[i + 1]]
        k = np.searchsorted(r, j)
        assert r[k] == j, (i, j)
        return off[i] + k

    es = sc.array("edge_slots").reshape(-1, 4)
    for e in range(sc._rod_count):
        a, b = (int(v) for v in E[e])
        assert list(es[e]) == [slot(a, a), slot(a, b), slot(b, a), slot(b, b)]
    bs = sc.array("rod_bend_slots").reshape(-1, 9)
    interior = 0
    for i in range(len(vm)):
        if len(ve[i]) == 2 and not vf[i]:
            st = [E[ve[i][0]][1] if E[ve[i][0]][0] == i else E[ve[i][0]][0], i,
                  E[ve[i][1]][1] if E[ve[i][1]][0] == i else E[ve[i][1]][0]]
            assert list(bs[i]) == [slot(int(a), int(b)) for a in st for b in st], i
            interior += 1
        else:
            assert np.all(bs[i] == 0xFFFFFFFF)
    assert interior == (24 - 2) + (16 - 2) + (12 - 2)


def test_rod_golden_matches_reference_build(ref_pipeline_or_none):
    """The frozen rod outputs are the reference's own, recomputed live where
    its sources are present."""
    ref = ref_pipeline_or_none
    if ref is None:
        pytest.skip("reference sources not present")
    import ctypes as C

    g = np.load(GOLDEN)
    sc, info = step_scenes.rods_and_sheet()
    prm = sc.param.contents
    assert ref.refpipe_init(sc.dataset, C.byref(prm))
    curr, prev = (a.reshape(-1).copy() for a in sc.positions())
    target = rpc.step_target(sc, curr, prev)
    assert np.array_equal(target, g["target"])
    dt = float(f32(prm.dt) * f32(prm.playback))
    keys, blocks, force, count = rpc.reference_first_system(ref, curr, prev, prm, target, dt)
    assert np.array_equal(keys, g["keys"]) and count == int(g["contacts"])
    assert np.array_equal(blocks.astype(f32), g["blocks"])
    assert np.array_equal(force, g["force"])
    assert ref.refpipe_rod_strain_line_search(curr, g["rod_ls_x1"]) == g["rod_ls"][0]


@pytest.mark.gpu
def test_rod_system_matches_reference(product_lib):
    """Every block and force entry of the product's first Newton system of
    the rods-and-sheet scene within 1e-5 of the reference's (each block
    against its diagonal scale), on an identical block pattern."""
    from oracle.binding import product_system

    g = np.load(GOLDEN)
    sc, info = step_scenes.rods_and_sheet()
    n = sc.vertex_count
    s = Session(sc)
    dx = np.zeros(3 * n, f32)
    it, rr = C.c_uint(), C.c_float()
    st = product_lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr))
    assert st == 0
    sysm = product_system(product_lib, n)
    keys, blocks = rpc.oracle_blocks(sysm, n)
    force = sysm["force"].reshape(-1).astype(np.float64)
    rpc.compare_systems(n, (g["keys"], g["blocks"].astype(np.float64), g["force"]),
                        (keys, blocks, force))
    del s


@pytest.mark.gpu
def test_rod_strain_line_search_matches_reference(product_lib):
    g = np.load(GOLDEN)
    sc, info = step_scenes.rods_and_sheet()
    s = Session(sc)
    curr = sc.positions()[0].reshape(-1).astype(f32)
    product_lib.ppf_debug_strain_line_search.restype = C.c_float
    product_lib.ppf_debug_strain_line_search.argtypes = [C.POINTER(C.c_float)] * 2
    x1 = np.ascontiguousarray(g["rod_ls_x1"])
    t = product_lib.ppf_debug_strain_line_search(
        curr.ctypes.data_as(C.POINTER(C.c_float)), x1.ctypes.data_as(C.POINTER(C.c_float)))
    assert t == g["rod_ls"][0], (t, g["rod_ls"][0])
    del s


@pytest.mark.gpu
def test_rod_trajectory_keeps_strain_limit(product_lib):
    """60 steps: every step succeeds, and every rod edge stays within its 1 %
    strain limit (plus the solver's line-search slack)."""
    sc, info = step_scenes.rods_and_sheet()
    E = sc.array("edge").reshape(-1, 2)[:sc._rod_count]
    l0 = sc.array("edge_initial_length")[:sc._rod_count]
    s = Session(sc)
    for k in range(60):
        r = s.step()
        assert r.success(), (k, r.as_dict())
        x = s.positions()
        assert np.all(np.isfinite(x))
        strain = np.linalg.norm(x[E[:, 1]] - x[E[:, 0]], axis=1) / l0 - 1.0
        assert strain.max() <= 0.01 + 1e-4, (k, strain.max())
    assert x[:, 1].min() >= 0.3 - 1e-6
