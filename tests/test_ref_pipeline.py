"""The oracle's Newton-system assembly, line searches and intersection check
against the reference's own code, on the CPU.

Live: oracle/_ref/libppfref_pipe.so is the reference's energy.cu,
strainlimiting.cu and contact.cu compiled as host code (oracle/Makefile); it
runs on the same states as the oracle. Frozen: tests/golden/ref_pipeline.npz
holds that library's outputs at the two-sheets scene's start state
(tests/golden/make_ref_pipeline.py), so hosts without the reference sources
still check the oracle against them.

Bars: the same block pattern; each block within 1e-5 of its diagonal scale
and the force within 1e-5 of its largest entry (fp32 sums in a different
order); the contact time of impact bit-exact; the strain-limit time of impact
bit-exact after the reference's division by line_search_max_t; the same
intersection verdicts.
"""
import ctypes as C

import numpy as np
import pytest

import ref_pipeline_cases as rpc
import step_scenes

GOLDEN = rpc.__file__.rsplit("/", 1)[0] + "/golden/ref_pipeline.npz"


@pytest.fixture(scope="module")
def scene(oracle_lib, product_lib):
    sc, _ = step_scenes.two_sheets()
    assert sc.vertex_count == 290  # the index ranges of ref_pipeline_cases
    return sc


@pytest.fixture(scope="module")
def ref_pipe():
    from oracle import binding
    from ppf_gb300 import build

    try:
        build.build_reference()
    except Exception:
        pass
    lib = binding.reference_pipeline()
    if lib is None:
        pytest.skip("reference sources not present on this host")
    return lib


def _session(scene):
    from oracle.binding import OracleSession

    return OracleSession(scene)


def _line_searches(o, x0, x1):
    pin, ov = C.c_uint(), C.c_int()
    toi = o.lib.oracle_line_search_at(x0, x1, C.byref(pin), C.byref(ov))
    strain = o.lib.oracle_strain_line_search_at(x0, x1)
    return toi, strain, pin.value, ov.value


def _check_line_searches(o, x0, dx, ref_of):
    """ref_of(name, x1) -> (ccd toi, strain toi, pin, overlap) of the reference."""
    T = np.float32(rpc.oracle_param(o).line_search_max_t)
    seen = {}
    for name, x1 in rpc.line_search_cases(x0, dx).items():
        toi, strain, pin, ov = _line_searches(o, x0, x1)
        r_toi, r_strain, r_pin, r_ov = ref_of(name, x1)
        assert np.float32(toi) == np.float32(r_toi), (name, toi, r_toi)
        assert np.float32(np.float32(strain) / T) == np.float32(r_strain), (name, strain, r_strain)
        assert (pin, ov) == (r_pin, r_ov), name
        seen[name] = (toi, strain / T)
    # the cases exercise what they are named for
    assert seen["sheet_b_down"][0] < 1.0 and seen["triangle_up"][0] < 1.0
    assert seen["stretch"][1] < 1.0


def test_assembly_matches_reference(scene, ref_pipe):
    o = _session(scene)
    assert ref_pipe.refpipe_init(scene.dataset, C.byref(o.param))
    for _ in range(rpc.STEPS):
        curr, prev, prm, target, dt, ok, ob, of = rpc.oracle_first_system(o)
        rk, rb, rf, count = rpc.reference_first_system(ref_pipe, curr, prev, prm, target, dt)
        rpc.compare_systems(o.n, (rk, rb, rf), (ok, ob, of))
        assert count > 0
        assert o.step().success()


def test_line_searches_and_intersection_match_reference(scene, ref_pipe):
    o = _session(scene)
    assert ref_pipe.refpipe_init(scene.dataset, C.byref(o.param))
    curr, prev, prm, *_ = rpc.oracle_first_system(o)
    ref_pipe.refpipe_state(curr, prev, C.byref(prm))
    _, dx, _, _ = o.newton_system()

    def ref_of(name, x1):
        pin, ov = C.c_uint(), C.c_int()
        toi = ref_pipe.refpipe_line_search(curr, x1, C.byref(pin), C.byref(ov))
        return toi, ref_pipe.refpipe_strain_line_search(curr, x1), pin.value, ov.value

    _check_line_searches(o, curr, dx.reshape(-1), ref_of)
    verdicts = {}
    for name, x in rpc.intersection_cases(curr).items():
        verdicts[name] = o.intersection_free(x)
        assert verdicts[name] == ref_pipe.refpipe_check_intersection(x), name
    assert verdicts == {"start": True, "tilted": False}


def test_oracle_matches_frozen_reference(scene):
    g = np.load(GOLDEN)
    o = _session(scene)
    curr, prev, prm, target, dt, ok, ob, of = rpc.oracle_first_system(o)
    rpc.compare_systems(o.n, (g["keys"], g["blocks"].astype(np.float64), g["force"]),
                        (ok, ob, of))
    # the frozen line searches ran along the frozen Newton direction
    dx = g["ls_dx"]

    def ref_of(name, x1):
        toi, strain = g[f"ls_{name}"]
        pin, ov = g[f"ls_{name}_flags"]
        return toi, strain, int(pin), int(ov)

    _check_line_searches(o, curr, dx, ref_of)
    for name, x in rpc.intersection_cases(curr).items():
        assert o.intersection_free(x) == bool(g[f"isect_{name}"]), name


def test_collision_mesh_matches_reference(oracle_lib, product_lib, ref_pipe):
    """A sheet inside the contact gap of a static collision box: the first
    Newton systems of 4 steps (cloth vertices against the box's faces, the
    box's corner against cloth faces) and the line searches of the sheet
    pushed into the box, against the reference's own collision-mesh code."""
    from oracle.binding import OracleSession

    sc, _ = step_scenes.cloth_on_box()
    o = OracleSession(sc)
    assert ref_pipe.refpipe_init(sc.dataset, C.byref(o.param))
    for _ in range(4):
        curr, prev, prm, target, dt, ok, ob, of = rpc.oracle_first_system(o)
        rk, rb, rf, count = rpc.reference_first_system(ref_pipe, curr, prev, prm, target, dt)
        rpc.compare_systems(o.n, (rk, rb, rf), (ok, ob, of))
        assert count > 40
        assert o.step().success()
    x0 = o.positions()[0].reshape(-1).copy()
    ref_pipe.refpipe_state(x0, o.positions()[1].reshape(-1).copy(),
                           C.byref(rpc.oracle_param(o)))
    for dy in (-3e-3, -3e-2):
        x1 = x0.reshape(-1, 3).copy()
        x1[:, 1] += dy
        x1 = x1.reshape(-1).astype(np.float32)
        pa, oa, pb, ob2 = C.c_uint(), C.c_int(), C.c_uint(), C.c_int()
        t_ref = ref_pipe.refpipe_line_search(x0, x1, C.byref(pa), C.byref(oa))
        t_orc = o.lib.oracle_line_search_at(x0, x1, C.byref(pb), C.byref(ob2))
        assert np.float32(t_ref) == np.float32(t_orc) and t_orc < 1.0, (dy, t_ref, t_orc)
        assert (pa.value, oa.value) == (pb.value, ob2.value)
    assert ref_pipe.refpipe_check_intersection(x0) and o.intersection_free(x0)


def test_twisted_tube_failure_is_the_reference_algorithm(oracle_lib, product_lib, ref_pipe):
    """A 32 x 64 twisted tube (both end rings pinned and turned at 2 rad/s)
    fails around step 65 with a non-finite Newton system, on the oracle as
    on the GPU. This pins that failure to the reference's own code: on the
    line-search inputs of the failing step's last Newton iterations (each
    admitting only a tiny step, the tube twisted against its 1% strain
    limit) the reference's strainlimiting::line_search returns the oracle's
    time of impact bit for bit, and the reference's own assembly at the
    iterate those steps reach holds non-finite blocks and forces (a face on
    the strain limit: the barrier's 1 / gap^2 stiffness)."""
    from oracle.binding import OracleSession
    from ppf_gb300 import abi, scenes

    sc, motion = scenes.twisted_tube(32, 64)
    o = OracleSession(sc, motion)
    failed = None
    for k in range(90):
        r = o.step()
        if not r.success():
            failed = (k, r.as_dict())
            break
    assert failed is not None and not failed[1]["pcg_success"], failed
    assert ref_pipe.refpipe_init(sc.dataset, C.byref(o.param))
    T = np.float32(o.param.line_search_max_t)
    records = [o.ls_trace(j) for j in range(8)]
    records = [r for r in records if r is not None]
    assert len(records) == 8
    for x0, x1, tc, ts in records:
        tref = ref_pipe.refpipe_strain_line_search(x0, x1)
        assert np.float32(np.float32(ts) / T) == np.float32(tref), (ts, tref)
        assert ts / T < 1e-3  # the strain limit admits a tiny step only
    # the iterate the newest record leads to, and the reference's system there
    x0, x1, tc, ts = records[0]
    toi = np.float32(min(tc, np.float32(ts) / T))
    ev = (x0 + (toi * (x1 - x0)).astype(np.float32)).astype(np.float32)
    curr, prev = o.positions()
    prm = abi.ParamSet.from_buffer_copy(o.param)
    prm.time = o.time
    ref_pipe.refpipe_state(curr.reshape(-1), prev.reshape(-1), C.byref(prm))
    ref_pipe.refpipe_assemble(ev, ev, np.float32(prm.dt))
    nb = ref_pipe.refpipe_blocks(None, None, None)
    rows, cols = np.zeros(nb, np.uint32), np.zeros(nb, np.uint32)
    blocks = np.zeros(9 * nb, np.float32)
    ref_pipe.refpipe_blocks(rows, cols, blocks)
    force = np.zeros(ev.size, np.float32)
    ref_pipe.refpipe_force(force)
    assert (~np.isfinite(blocks)).sum() > 0 and (~np.isfinite(force)).sum() > 0
