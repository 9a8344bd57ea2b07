import sys, tempfile, pathlib, subprocess
sys.path.insert(0, "tests"); sys.path.insert(0, "ppf-contact-solver_gb300"); sys.path.insert(0, ".")
import numpy as np
import test_driver as td
from ppf_gb300 import scenes, session_io, build
from ppf_gb300.session import Scene, Session, RodMaterial

build.build_driver()
tmp = pathlib.Path(tempfile.mkdtemp())
path, verts, f, rod = td._rod_session(tmp, frames=6)
out = tmp / "out"
r = subprocess.run([str(session_io.executable()), "--path", str(path), "--output", str(out)], capture_output=True, text=True)
print("driver rc", r.returncode, r.stderr[-300:])
v, _ = td._scene_arrays(8)

def python_traj(with_stitch=True):
    sc = Scene()
    sc.add_shell(v.astype(np.float32), f, scenes.cloth_material())
    sc.add_rod(verts[len(v):].astype(np.float32), rod - len(v), RodMaterial(density=0.01, young_mod=1e4, bend=0.5, strain_limit=0.01, contact_gap=1e-3, friction=0.3))
    sc.add_floor((0.0, 0.0, 0.0), contact_gap=1e-3, friction=0.5)
    if with_stitch:
        for e in [len(v), len(v) + len(rod)]:
            m = int(np.argmin(np.linalg.norm(v - verts[e], axis=1)))
            sc.add_stitch([e, e, e, m, m, m], [1, 0, 0, 1, 0, 0], 0.5)
    sc.build(scenes._param(0.01))
    s = Session(sc)
    traj, times, toi = [sc.positions()[0].copy()], [0.0], []
    while times[-1] < 6 / td.FPS:
        res = s.step()
        assert res.success()
        traj.append(s.positions().copy()); times.append(s.time)
        toi.append(list(s.stats().toi[: s.stats().newton_iters]) if hasattr(s.stats(), "toi") else None)
    return traj, times

t1, s1 = python_traj(); t2, s2 = python_traj()
print("times1", [round(t, 5) for t in s1]); print("times2", [round(t, 5) for t in s2])
for k in range(7):
    a = td._interp(t1, s1, k / td.FPS); b = td._interp(t2, s2, k / td.FPS)
    d = session_io.read_frame(out, k)
    print(k, "py-py", float(np.abs(a - b).max()), "drv-py", float(np.abs(d - a).max()))
