"""The solver executable (csrc/driver/main.cpp) on scene directories in the
reference's session format.

CPU: the executable reads a written scene back (--describe): counts of
vertices, faces, pins, colliders and the collision mesh, and the [param]
values, with the step clamped below one frame as the reference does
(builder.rs:273-275).

GPU: frames written by the executable are the library's own trajectory of
the same scene (stepped through the Python session), interpolated to the
frame times; a run resumed from a checkpoint reproduces the frames after it.
"""
import shutil
import subprocess

import numpy as np
import pytest

from ppf_gb300 import meshes, scenes, session_io
from ppf_gb300.session import Scene, Session

FPS = 60.0


def _scene_arrays(side=16):
    v, f = meshes.grid(side, side, 0.6, 0.6)
    v = v.astype(np.float64)
    v[:, 1] = 0.45
    return v, f


def _session(tmp_path, side=16, frames=8, auto_save=4, with_mesh=True):
    v, f = _scene_arrays(side)
    mat = scenes.cloth_material()
    nf = len(f)
    fp = {"model": np.full(nf, 2, np.uint8), "density": np.full(nf, mat.density),
          "young-mod": np.full(nf, mat.young_mod), "poiss-rat": np.full(nf, mat.poiss_rat),
          "bend": np.full(nf, mat.bend), "strain-limit": np.full(nf, mat.strain_limit),
          "contact-gap": np.full(nf, mat.contact_gap),
          "contact-offset": np.full(nf, mat.contact_offset),
          "friction": np.full(nf, mat.friction)}
    bv, bf = meshes.box(0.2, center=(0.15, 0.1, 0.0))
    sc = session_io.SessionScene(
        vert=v, tri=f, face_params=fp,
        pins=[(np.array([0]), 0.0)],
        walls=[session_io.Wall(position=(0.0, 0.0, 0.0), contact_gap=1e-3, friction=0.5)],
        spheres=[session_io.Sphere(center=(-0.15, 0.1, 0.0), radius=0.12, contact_gap=1e-3,
                                   friction=0.5)],
        static_vert=bv if with_mesh else None, static_tri=bf if with_mesh else None,
        static_params={"contact-gap": np.full(len(bf), 1e-3), "friction": np.full(len(bf), 0.5)},
        param={"dt": 0.01, "frames": frames, "fps": FPS, "auto_save": auto_save,
               "gravity": [0.0, -9.8, 0.0], "cg_tol": 1e-3})
    return session_io.write_session(tmp_path / "scene", sc)


def _python_scene(side=16, with_mesh=True):
    """The same scene through the Python builder API."""
    v, f = _scene_arrays(side)
    sc = Scene()
    sc.add_shell(v.astype(np.float32), f, scenes.cloth_material())
    sc.pin([0])
    sc.add_sphere((-0.15, 0.1, 0.0), 0.12, contact_gap=1e-3, friction=0.5)
    sc.add_floor((0.0, 0.0, 0.0), contact_gap=1e-3, friction=0.5)
    if with_mesh:
        bv, bf = meshes.box(0.2, center=(0.15, 0.1, 0.0))
        sc.add_collision_mesh(bv, bf, contact_gap=1e-3, friction=0.5)
    return sc.build(scenes._param(0.01))


def _run(args, timeout=600):
    return subprocess.run([str(session_io.executable()), *map(str, args)],
                          capture_output=True, text=True, timeout=timeout)


@pytest.fixture(scope="module")
def driver(product_lib):
    from ppf_gb300 import build

    build.build_driver()
    return session_io.executable()


def test_driver_reads_the_session_format(driver, tmp_path):
    path = _session(tmp_path)
    r = _run(["--path", path, "--describe"])
    assert r.returncode == 0, r.stderr
    d = {}
    for line in r.stdout.splitlines():
        k, *v = line.split()
        d[k] = [float(x) for x in v]
    v, f = _scene_arrays()
    bv, bf = meshes.box(0.2)
    assert d["vertices"] == [len(v)] and d["faces"] == [len(f)]
    assert d["fix"] == [1] and d["pull"] == [0]
    assert d["spheres"] == [1] and d["floors"] == [1]
    assert d["collision_vertices"] == [len(bv)] and d["collision_faces"] == [len(bf)]
    assert d["face_params"] == [1]  # one material, deduplicated
    assert d["frames"] == [8] and d["fps"] == [FPS] and d["auto_save"] == [4]
    assert d["gravity"] == [0.0, pytest.approx(-9.8), 0.0]
    assert d["dt"] == [pytest.approx(0.01)]
    # a step never spans a frame: dt is clamped to 0.9999 / fps
    (path / "param.toml").write_text(
        (path / "param.toml").read_text().replace("fps = 60.0", "fps = 200.0"))
    d2 = _run(["--path", path, "--describe"]).stdout
    assert f"dt {0.9999 / 200.0:.9g}"[:9] in d2


def test_driver_refuses_what_it_does_not_simulate(driver, tmp_path):
    path = _session(tmp_path)
    info = (path / "info.toml").read_text()
    (path / "info.toml").write_text(info.replace("tet = 0", "tet = 3"))
    r = _run(["--path", path, "--describe"])
    assert r.returncode == 1 and "tets" in r.stderr


def _interp(traj, times, t):
    for k in range(1, len(times)):
        if times[k] >= t - 1e-12:
            a = (t - times[k - 1]) / (times[k] - times[k - 1])
            return traj[k - 1] + np.float32(a) * (traj[k] - traj[k - 1])
    raise AssertionError(t)


@pytest.mark.gpu
def test_driver_frames_follow_the_library_trajectory(driver, tmp_path):
    path = _session(tmp_path, frames=8, auto_save=4)
    out = tmp_path / "out"
    r = _run(["--path", path, "--output", out])
    assert r.returncode == 0, r.stderr + r.stdout
    assert (out / "finished.txt").exists()
    for k in range(9):
        assert (out / f"vert_{k}.bin").exists(), k
    assert (out / "state_4.bin").exists() and (out / "state_8.bin").exists()
    assert (out / "data" / "advance.newton_steps.out").exists()
    # the same scene stepped through the session API, frames interpolated
    sc = _python_scene()
    s = Session(sc)
    traj, times = [sc.positions()[0].copy()], [0.0]
    while times[-1] < 8 / FPS:
        assert s.step().success()
        traj.append(s.positions().copy())
        times.append(s.time)
    # two runs of the library differ by the order of the atomic sums in the
    # assembly, which the 1e-3 relative PCG residual carries into each step:
    # frames agree to that fraction of the motion so far (the cloth falls
    # freely over these frames)
    for k in range(9):
        got = session_io.read_frame(out, k)
        want = _interp(traj, times, k / FPS)
        moved = float(np.abs(want - traj[0]).max())
        assert np.abs(got - want).max() <= 1e-3 * moved + 1e-7, (k, np.abs(got - want).max(),
                                                                 moved)
    # frame_to_time holds the exact frame times
    ft = np.loadtxt(out / "data" / "frame_to_time.out")
    assert np.allclose(ft[:, 1], ft[:, 0] / FPS, atol=1e-9)


@pytest.mark.gpu
def test_driver_resumes_from_a_checkpoint(driver, tmp_path):
    path = _session(tmp_path, frames=10, auto_save=5)
    out = tmp_path / "out"
    r = _run(["--path", path, "--output", out])
    assert r.returncode == 0, r.stderr + r.stdout
    first = {k: session_io.read_frame(out, k) for k in range(6, 11)}
    resumed = tmp_path / "resumed"
    shutil.copytree(out, resumed)
    for k in range(6, 11):
        (resumed / f"vert_{k}.bin").unlink()
    r = _run(["--path", path, "--output", resumed, "--load", "5"])
    assert r.returncode == 0, r.stderr + r.stdout
    start = session_io.read_frame(out, 5)
    for k in range(6, 11):
        got = session_io.read_frame(resumed, k)
        moved = float(np.abs(first[k] - start).max())
        assert np.abs(got - first[k]).max() <= 1e-3 * moved + 1e-7, (
            k, np.abs(got - first[k]).max(), moved)
    # --load -1 resumes from the latest checkpoint
    r = _run(["--path", path, "--output", resumed, "--load", "-1"])
    assert r.returncode == 0, r.stderr


def _rod_session(tmp_path, frames=6):
    """A sheet and a rod above it, written with per-rod parameter arrays."""
    v, f = _scene_arrays(8)
    nr = 10
    rv = np.stack([np.linspace(-0.2, 0.2, nr), np.full(nr, 0.46), np.full(nr, 0.01)], 1)
    verts = np.concatenate([v, rv])
    rod = np.stack([np.arange(nr - 1), np.arange(1, nr)], 1) + len(v)
    mat = scenes.cloth_material()
    nf = len(f)
    fp = {"density": np.full(nf, mat.density), "young-mod": np.full(nf, mat.young_mod),
          "poiss-rat": np.full(nf, mat.poiss_rat), "bend": np.full(nf, mat.bend),
          "strain-limit": np.full(nf, mat.strain_limit),
          "contact-gap": np.full(nf, mat.contact_gap), "friction": np.full(nf, mat.friction)}
    r = nr - 1
    rp = {"density": np.full(r, 0.01), "young-mod": np.full(r, 1e4), "bend": np.full(r, 0.5),
          "length-factor": np.full(r, 1.0), "strain-limit": np.full(r, 0.01),
          "contact-gap": np.full(r, 1e-3), "friction": np.full(r, 0.3)}
    # the rod's ends stitched to the sheet's nearest vertices
    ends = [len(v), len(v) + nr - 1]
    near = [int(np.argmin(np.linalg.norm(v - verts[e], axis=1))) for e in ends]
    sind = np.array([[e, e, e, m, m, m] for e, m in zip(ends, near)], np.uint64)
    sw = np.tile(np.array([1, 0, 0, 1, 0, 0], np.float32), (2, 1))
    sc = session_io.SessionScene(
        vert=verts, tri=f, face_params=fp, rod=rod, rod_params=rp,
        stitch_ind=sind, stitch_w=sw, stitch_stiffness=np.full(2, 1e-6, np.float32),
        walls=[session_io.Wall(position=(0.0, 0.0, 0.0), contact_gap=1e-3, friction=0.5)],
        param={"dt": 0.01, "frames": frames, "fps": FPS, "auto_save": 0,
               "gravity": [0.0, -9.8, 0.0], "cg_tol": 1e-3})
    return session_io.write_session(tmp_path / "rods", sc), verts, f, rod


def test_driver_reads_rods(driver, tmp_path):
    path, verts, f, rod = _rod_session(tmp_path)
    r = _run(["--path", path, "--describe"])
    assert r.returncode == 0, r.stderr
    d = dict(line.split(maxsplit=1) for line in r.stdout.splitlines())
    assert int(d["vertices"]) == len(verts) and int(d["faces"]) == len(f)
    assert int(d["rods"]) == len(rod) and int(d["stitches"]) == 2
    assert int(d["edges"]) > len(rod)  # the rod edges, then the faces' edges


@pytest.mark.gpu
def test_driver_rod_frames_follow_the_library(driver, tmp_path):
    """A session with a rod: the executable's frames are the library's
    trajectory of the same scene built through the Python API."""
    from ppf_gb300.session import RodMaterial

    path, verts, f, rod = _rod_session(tmp_path, frames=6)
    out = tmp_path / "out"
    r = _run(["--path", path, "--output", out])
    assert r.returncode == 0, r.stderr + r.stdout
    sc = Scene()
    v, _ = _scene_arrays(8)
    sc.add_shell(v.astype(np.float32), f, scenes.cloth_material())
    sc.add_rod(verts[len(v):].astype(np.float32), rod - len(v),
               RodMaterial(density=0.01, young_mod=1e4, bend=0.5, strain_limit=0.01,
                           contact_gap=1e-3, friction=0.3))
    sc.add_floor((0.0, 0.0, 0.0), contact_gap=1e-3, friction=0.5)
    ends = [len(v), len(v) + len(rod)]
    for e in ends:
        m = int(np.argmin(np.linalg.norm(v - verts[e], axis=1)))
        sc.add_stitch([e, e, e, m, m, m], [1, 0, 0, 1, 0, 0], 1e-6)
    sc.build(scenes._param(0.01))
    curr0, prev0 = sc.positions()

    def trajectory():
        sc.set_positions(curr0, prev0)
        sc.param.contents.time = 0.0
        s = Session(sc)
        traj, times = [curr0.copy()], [0.0]
        while times[-1] < 6 / FPS:
            assert s.step().success()
            traj.append(s.positions().copy())
            times.append(s.time)
        return traj, times

    # the rod falls 1 cm above the sheet, its ends held to it by weak
    # stitches; two runs of the library differ by the order of the assembly's
    # atomic sums carried through the PCG tolerance. The executable's frames
    # must stay within twice that run-to-run spread of the library's
    # trajectory.
    (t1, s1), (t2, s2) = trajectory(), trajectory()
    for k in range(7):
        got = session_io.read_frame(out, k)
        a, b = _interp(t1, s1, k / FPS), _interp(t2, s2, k / FPS)
        spread = float(np.abs(a - b).max())
        d = float(min(np.abs(got - a).max(), np.abs(got - b).max()))
        assert d <= 2.0 * spread + 1e-5, (k, d, spread)
