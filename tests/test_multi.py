"""Many scenes stepped together (ppf_multi_*): each scene's trajectory is
the one the same scene takes stepped alone with the same PCG team, up to the
order of the float atomics in the assembly; every scene gets the PCG team
its size asks for."""
import ctypes as C

import numpy as np
import pytest

import step_scenes
from ppf_gb300 import scenes
from ppf_gb300.multi import MultiSession
from ppf_gb300.session import Session

pytestmark = pytest.mark.gpu

DROPS = scenes.uneven_drops(8, seed=3)


def _build(p):
    side, height, collider, size = p
    sc, _ = scenes.cloth_drop(side, height, collider, size)
    return sc


def _team(n):
    """The PCG team ppf_multi_create gives a scene of n vertices."""
    return 2 if n <= 2048 else 4 if n <= 4096 else 8 if n <= 8192 else 16 if n <= 16384 else 0


def _alone(sc, motion=None):
    """A session on the scene with the PCG team (and CTA size) the
    multi-scene solver gives it, so the two run the same reductions."""
    s = Session(sc, motion) if motion is not None else Session(sc)
    s.lib.ppf_set_pcg_team.argtypes = [C.c_int]
    s.lib.ppf_set_pcg_cta_threads.argtypes = [C.c_uint]
    assert s.lib.ppf_set_pcg_team(_team(sc.vertex_count)) == 0
    assert s.lib.ppf_set_pcg_cta_threads(512) == 0
    return s


def _alone_runs(make, steps, runs=3):
    """Positions after steps + 1 steps of `runs` sessions on the same scene,
    each alone with the multi-scene PCG team, with (their largest pairwise
    difference, the largest displacement of the run): the library's own
    run-to-run spread (the assembly's float atomics add in an order that
    varies from run to run) and the motion it is relative to."""
    xs = []
    for _ in range(runs):
        sc, motion = make()
        x0 = sc.positions()[0].copy()
        s = _alone(sc, motion)
        for _ in range(steps):
            assert s.step(fetch=False).success()
        s.step()
        xs.append(s.positions().copy())
        del s, sc
    spread = max(np.abs(a - b).max() for i, a in enumerate(xs) for b in xs[i + 1:])
    return xs[0], (spread, np.abs(xs[0] - x0).max())


def _close(x, ref, bound):
    """Within a few times the run-to-run spread, or within what the 1e-3
    relative PCG residual leaves of the motion (1e-3 of the largest
    displacement over the run), never tighter than 1e-5 relative."""
    spread, disp = bound
    return np.abs(x - ref).max() <= max(3.0 * spread, 1e-3 * disp, 1e-5 * np.abs(ref).max())


def test_multi_matches_scenes_stepped_alone(product_lib):
    steps = 12
    alone = [_alone_runs(lambda p=p: (_build(p), None), steps) for p in DROPS]
    built = [_build(p) for p in DROPS]
    m = MultiSession(built, threads=4)
    for k in range(steps + 1):
        res = m.step()
        assert all(r.success() for r in res), k
    for i, p in enumerate(DROPS):
        x = m.positions(i)
        ref, bound = alone[i]
        assert _close(x, ref, bound), (i, p, np.abs(x - ref).max(), bound)
        st = m.stats(i)
        assert st.newton_iters >= 1 and st.vertices == built[i].vertex_count
        assert m.pcg_team(i) == _team(built[i].vertex_count)
    m.close()


def test_multi_rejects_an_intersecting_scene(product_lib):
    """A scene that starts self-intersecting fails its create; the handle is
    not made and the fatal detail names the scene."""
    from ppf_gb300 import meshes

    good = _build(DROPS[0])
    v, f = meshes.grid(8, 8, 1.0, 1.0)
    v2 = v.copy()
    v2[:, 1] = 0.0
    v3 = v.copy()
    v3[:, [0, 1, 2]] = v3[:, [1, 0, 2]]  # a vertical sheet through the first
    sc = scenes.Scene()
    sc.add_shell(np.concatenate([v2, v3]), np.concatenate([f, f + len(v)]),
                 scenes.cloth_material())
    bad, _ = sc.build(scenes._param(0.01)), None
    with pytest.raises(Exception):
        MultiSession([good, bad], threads=2)


def test_multi_pinned_moving_scenes(product_lib):
    """Twisted tubes (both end rings pinned and turned) stepped together with
    their pin motions follow the same tubes stepped alone."""
    steps = 6
    makers = [lambda: scenes.twisted_tube(16, 24), lambda: scenes.twisted_tube(24, 32)]
    alone = [_alone_runs(make, steps) for make in makers]
    built = [make() for make in makers]
    m = MultiSession([b[0] for b in built], threads=2, pin_motions=[b[1] for b in built])
    for _ in range(steps + 1):
        assert all(r.success() for r in m.step())
    for i in range(len(makers)):
        x = m.positions(i)
        ref, bound = alone[i]
        assert _close(x, ref, bound), (i, np.abs(x - ref).max(), bound)
    m.close()


def test_multi_step_matches_the_oracle(product_lib):
    """Two contact scenes (the two sheets after three oracle steps, pinned and
    unpinned) stepped together: each scene's step matches the oracle's step
    from the same state within 1e-5 relative, as a scene stepped alone does.
    The oracle holds one scene at a time, so each scene's oracle step is
    taken before the next scene is built."""
    from oracle.binding import OracleSession

    states, expect = [], []
    for pinned in (True, False):
        sc, _ = step_scenes.two_sheets(pinned=pinned)
        orc = OracleSession(sc)
        for _ in range(3):
            assert orc.step().success()
        curr, prev = orc.positions()
        t = orc.time
        sc.set_positions(curr, prev)
        sc.param.contents.time = t
        o = OracleSession(sc)
        assert o.step().success()
        expect.append(o.positions()[0].copy())
        states.append((pinned, curr.copy(), prev.copy(), t))
        del o, orc, sc
    built = []
    for pinned, curr, prev, t in states:
        sc, _ = step_scenes.two_sheets(pinned=pinned)
        sc.set_positions(curr, prev)
        sc.param.contents.time = t
        built.append(sc)
    m = MultiSession(built, threads=2)
    res = m.step()
    assert all(r.success() for r in res)
    for i, xo in enumerate(expect):
        xg = m.positions(i)
        assert np.abs(xg - xo).max() <= 1e-5 * np.abs(xo).max(), (i, np.abs(xg - xo).max())
    m.close()
